"""Benchmark of the GB300 DEM timestep (particle-steps/s), one JSON line on rank 0.

Workloads (synthetic, seeded; no dataset is involved):
  hertz1M (default) -- 1,000,000 polydisperse HertzMat spheres (r ~ U[2,6] mm, DMT, en=.8, surfEnergy
      .01, tanPhi .3/.6) as a loose cloud (solid fraction ~0.3) falling into a 1 x 1 x 2 m walled box,
      dt = 0.3 x p-wave dt, verletDist 0.1 x rmin.  The timed region is K steps after W warm-up steps of
      that job, the same steps that the CPU arm (--impl reference) times.  The line also carries
      "settled": the same spheres settled on the GPU first (untimed, damping 0.5: 10 g while the cloud
      falls, then 1 g; scenes.settle), then W + K steps with the job's parameters, about one real contact
      per sphere, with the CPU port timed on that same settled state in the same process.
  hertz1M_settled -- the settled state alone as the headline.
  ell200k -- 200,000 ellipsoids (a ~ U[3,6] mm, b = .7a, c = .5a, random orientations) agitated in a
      0.6 x 0.6 x 1.2 m walled box under gravity, FrictMat E 1e7 tanPhi .4, dt 0.9 x p-wave dt.  The
      learned warm start is trained first (untimed) on records logged by the plain Newton solver; the
      line reports the learned-warm-start run and, under "variants", the reference's Brent solver, the
      plain cold-start Newton and the previous-step warm start on the same initial state.
  batch512 -- 512 independent oedometric scenes (sphere counts log-uniform in [500, 20000], r ~ U[1,3] mm,
      tanPhi ~ U[.1,.8], young log-uniform in [1e6,1e8] Pa, per-scene dt, top wall at 0.05 m/s) stepped
      as one batch; "scene_by_scene" times a seeded sample of 32 of the scenes run one after another on
      their own handles and scales it to all 512.
  peri8M -- 8,000,000 spheres, lognormal radii (median 1 mm, sigma .25, clipped [.5,2] mm) in a periodic
      cell under simple shear (gradV rate 1/s), FrictMat E 1e8 tanPhi .5, IdealElPl; packed by periodic
      random sequential addition at solid fraction 0.3, then densified to 0.62 on the GPU (radius growth
      with damping, scaled back to the original radii; untimed); the stress tensor at the
      end of the timed steps is reported.
  spheres10k -- 10,000 monodisperse FrictMat spheres r = 5 mm in a 0.5 x 0.5 x 1 m box (CPU-runnable).

A step is one pass of the hot path (Leapfrog -> collider -> ContactLoop) over all particles; the timed
region covers K consecutive steps of one simulation, state resident in HBM (larger than L2).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--workload ...]

--impl reference times the reference algorithm on the host cores: the OpenMP build of the CPU
restatement of Woo's Leapfrog/InsertionSortCollider/ContactLoop, on the same scene (built by the
oracle's copy of the packing generator, so the engine library is never loaded) and the same W + K steps.
Multi-GPU: the path does not shard (contacts couple neighbours); N ranks run N independent replicas.
"""
import argparse
import ctypes
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np

WORKLOADS = ["hertz1M", "hertz1M_settled", "ell200k", "batch512", "peri8M", "spheres10k"]
DEFAULT_STEPS = {"hertz1M": 20, "hertz1M_settled": 20, "ell200k": 500, "batch512": 500, "peri8M": 500,
                 "spheres10k": 2000}
METRIC = "particle-steps/s per GB300"
DESCR = {"hertz1M": "plain DEM step, HertzDMT settling",
         "hertz1M_settled": "plain DEM step, HertzDMT, settled packing",
         "ell200k": "ellipsoid DEM step, learned warm start",
         "batch512": "512 batched oedometric scenes",
         "peri8M": "periodic simple shear, FrictMat IdealElPl",
         "spheres10k": "plain DEM step, FrictMat IdealElPl"}


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default: per workload)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="hertz1M", choices=WORKLOADS)
    ap.add_argument("--e2e-steps", type=int, default=2000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--queue-depth", type=int, default=None,
                    help="steps queued before the host checks the collider trigger (engine default 32; 1 = every step)")
    ap.add_argument("--n", type=int, default=None,
                    help="particle count of a smaller cut of the workload (same density; for profiling runs)")
    ap.add_argument("--no-settled", action="store_true", help="hertz1M: leave out the settled-state object")
    ap.add_argument("--arith", default="fma", choices=["fma", "dw", "exact"],
                    help="arithmetic of the contact and integrator kernels (wdem_params.arith): FP64 with FMA "
                         "contraction, that with the contact law in double-word FP32, or the reference's IEEE "
                         "operations bit for bit")
    ap.add_argument("--autotune", default="auto", choices=["auto", "on", "off"],
                    help="tune the kernels' launch shape (wdem_autotune) before the timed region; auto: batch512 only")
    ap.add_argument("--graphs", default="off", choices=["auto", "on", "off"],
                    help="queued steps launched as CUDA graphs (wdem_set_step_graphs): off (default), auto, on")
    ap.add_argument("--profile-region", default="main", choices=["main", "settled", "none"],
                    help="timed region bracketed by cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    a = ap.parse_args()
    if a.steps is None:
        a.steps = DEFAULT_STEPS[a.workload]
    return a


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def load_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1])); smax.append(float(f[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if f[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_scene(name, n=None, packer="engine"):
    """The workload's seeded scene.  packer="oracle" builds the same packing with the oracle's restatement
    of the generator (the CPU arm, which must not load the engine library)."""
    from woo_gb300 import abi, scenes
    if packer == "oracle":
        from oracle import bridge
        scenes.set_packer(bridge.make_cloud, bridge.make_cloud_radii)
    try:
        if name == "hertz1M":
            return scenes.hertz1M(n=n or 1_000_000)
        if name == "hertz1M_settled":
            return scenes.hertz1M(n=n or 1_000_000, height=0.95)
        if name == "peri8M":
            return scenes.densify_periodic(scenes.peri_shear(n=n or 8_000_000), phi_target=0.62)
        if name == "batch512":
            return scenes.batch_oedometric(n or 512, 4)
        if name == "ell200k":
            k = n or 200_000
            sc = (k / 200_000) ** (1.0 / 3.0)
            return scenes.ellipsoid_cloud(k, 7, box=(0.6 * sc, 0.6 * sc, 1.2 * sc), amin=0.003, amax=0.006, dense=1.0,
                                          vel_scale=0.5, angvel_scale=5.0, young=1e7, tanPhi=0.4, damping=0.2,
                                          ellSolver=abi.ELL_NEWTON, warmStart=abi.WARM_HISTORY_MLP)
        return scenes.spheres10k(n=n or 10000)
    finally:
        scenes.set_packer()


def copy_params(p):
    from woo_gb300 import scenes
    return scenes.copy_params(p)


def settle(h, spec):
    """Untimed settling on the GPU (scenes.settle): damping 0.5, 10 g while the cloud falls, then 1 g; the
    job's parameters are restored."""
    from woo_gb300 import scenes
    return scenes.settle(h, spec)


def contact_kernel_bytes(cg, hertz):
    """Algorithmic bytes of one contact pass (fixed per-unit figures): 80 B per particle touched by a real
    contact (pos 24, vel 24, angVel 24, radius 8), 288 B per real contact (ids 8, history read 112, history
    write 96, reduction outputs 72; Hertz adds 16 B r/w of kn, kt and 8 B contRad), 16 B per live
    potential-only pair (ids 8 + the distance-test data 8)."""
    live = cg.n
    r = cg.real == 1
    real = int(r.sum())
    pot = live - real
    touched = len(np.unique(np.concatenate([cg.idA[r], cg.idB[r]]))) if real else 0
    per_real = 288 + (24 if hertz else 0)
    return 80 * touched + per_real * real + 16 * pot, dict(real=real, potential=pot, touched_by_real=touched)


def max_over_ranks(x, world, device):
    """The largest of the ranks' values (the slowest rank's time): all-reduce MAX when world > 1."""
    import torch
    t = torch.tensor([x], device=device, dtype=torch.float64)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(world, n, steps, seconds):
    """Whole-job particle-steps/s of `world` replicas of an n-particle scene stepped `steps` times, timed
    by the slowest replica."""
    return world * n * steps / seconds


def timed_steps(h, stream, k, world, local, barrier, profile=False):
    """K steps timed with CUDA events on the engine's stream (barrier and synchronize on both sides); with
    profile, the region is bracketed by cudaProfilerStart/Stop for ncu --profile-from-start off."""
    import torch
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    if profile:
        torch.cuda.profiler.start()
    ev0.record(stream)
    h.step(k)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    if profile:
        torch.cuda.profiler.stop()
    barrier()
    ms = ev0.elapsed_time(ev1)
    return max_over_ranks(ms, world, f"cuda:{local}")


QUEUE_DEPTH = None
GRAPHS = "off"


def new_handle(spec, local, params=None):
    from woo_gb300 import abi
    h = abi.Handle(spec.particles.n, device=local)
    if QUEUE_DEPTH is not None:
        h.set_queue_depth(QUEUE_DEPTH)
    h.set_step_graphs({"auto": abi.GRAPHS_AUTO, "on": abi.GRAPHS_ON, "off": abi.GRAPHS_OFF}[GRAPHS])
    h.set_params(params or spec.params)
    h.upload_particles(spec.particles)
    h.set_params(params or spec.params)
    if getattr(spec, "cell", None) is not None:
        h.set_cell(**spec.cell)
    return h


def ell_variants(args, spec, local, world, barrier, w):
    """The same initial state under each solver: Brent (the reference's), Newton from the cold start,
    Newton from the previous step's lambda, Newton from the learned warm start (weights w), and Newton
    from the previous step's lambda with the learned warm start for pairs solved for the first time."""
    import torch
    from woo_gb300 import abi
    out = {}
    for name, solver, warm in (("brent", abi.ELL_BRENT, abi.WARM_COLD), ("newton_cold", abi.ELL_NEWTON, abi.WARM_COLD),
                               ("newton_history", abi.ELL_NEWTON, abi.WARM_HISTORY),
                               ("newton_mlp", abi.ELL_NEWTON, abi.WARM_MLP),
                               ("newton_history_mlp", abi.ELL_NEWTON, abi.WARM_HISTORY_MLP)):
        p = copy_params(spec.params)
        p.ellSolver, p.warmStart = solver, warm
        h = new_handle(spec, local, p)
        if warm in (abi.WARM_MLP, abi.WARM_HISTORY_MLP):
            h.warm_set_weights(w)
        stream = torch.cuda.ExternalStream(h.stream(), device=local)
        h.step(max(args.warmup, 3))
        s0 = h.status()
        h.set_timing(True)
        ms = timed_steps(h, stream, args.steps, world, local, barrier)
        kt = h.kernel_times()
        s1 = h.status()
        h.set_timing(False)
        solves = s1.ellSolves - s0.ellSolves
        c_ms, c_n = kt.get("contacts", (0.0, 1))
        out[name] = {"value": world * spec.particles.n * args.steps / (ms / 1e3), "ms_per_step": ms / args.steps,
                     "contacts_ms_per_step": c_ms / max(c_n, 1), "solves_per_step": solves / args.steps,
                     "iterations_per_solve": (s1.ellIters - s0.ellIters) / max(solves, 1),
                     "fallback_fraction": (s1.ellFallbacks - s0.ellFallbacks) / max(solves, 1)}
        h.close()
    return out


def state_tag(args, region, n):
    """Descriptor of the state a timed region starts from; an ncu summary under profiles/ is used for this
    region's traffic only when it records the same descriptor (a capture of the same deterministic run)."""
    tag = f"{args.workload}/{region}/n={n}/warmup={max(args.warmup, 3)}/steps={args.steps}"
    return tag if args.arith == "fma" else f"{tag}/arith={args.arith}"


def read_profile_figures(tag):
    """`- name: number` figures of the ncu summary under profiles/ that records `- state: <tag>`."""
    d = os.path.join(ROOT, "profiles")
    if not os.path.isdir(d):
        return {}
    for fn in sorted(os.listdir(d)):
        if not fn.endswith(".md"):
            continue
        figs, st = {}, None
        with open(os.path.join(d, fn)) as f:
            for line in f:
                m = re.match(r"^- state: (\S+)\s*$", line)
                if m:
                    st = m.group(1)
                m = re.match(r"^- ([\w.]+): ([0-9.eE+-]+)\s*$", line)
                if m:
                    figs[m.group(1)] = float(m.group(2))
        if st == tag:
            return figs
    return {}


PHASE_KERNELS = {"contacts": ("k_contacts_cull", "k_contacts"), "leapfrog": ("k_leapfrog_fast", "k_leapfrog_lists")}
PHASE_LABEL = {"contacts": "contact pass (k_contacts_cull + k_contacts: Cg2+Cp2+Law2)",
               "leapfrog": "integrator (k_leapfrog_fast + k_leapfrog_lists: CSR force gather + Leapfrog + verlet check)"}


def measure_region(h, spec, args, world, local, barrier, region, clocks=None):
    """W warm-up steps, K timed steps (CUDA events), then a window of steps with per-phase CUDA events for
    the roofline objects and the collider figures.  Returns the region's figures."""
    import torch
    from woo_gb300 import abi
    n = spec.particles.n
    stream = torch.cuda.ExternalStream(h.stream(), device=local)
    h.step(max(args.warmup, 3))
    st0 = h.status()
    l0 = h.launch_count()
    g0 = h.graph_stats()
    ms = timed_steps(h, stream, args.steps, world, local, barrier, profile=(args.profile_region == region))
    launches = h.launch_count() - l0
    g1 = h.graph_stats()
    st1 = h.status()
    cg = h.download_contacts()   # the state at the end of the timed region
    hertz = spec.params.cp2 == abi.CP2_HERTZ
    cbytes, counts = contact_kernel_bytes(cg, hertz)
    lbytes = 256 * n + 80 * counts["real"]   # Leapfrog 300 + CSR 52 - 96 fused B/particle, 80 B/real contact
    # per-phase CUDA events over a following window (the timed region runs without them)
    kw = max(args.steps, 200)
    s0 = h.status()
    h.set_timing(True)
    torch.cuda.synchronize()
    h.step(kw)
    torch.cuda.synchronize()
    kt = h.kernel_times()
    h.set_timing(False)
    s1 = h.status()
    hbm_peak, peak_kind = load_peaks()
    fp64_peak = h.fp64_peak()
    figs = read_profile_figures(state_tag(args, region, n))
    rl = {}
    for ph, abytes in (("contacts", cbytes), ("leapfrog", lbytes)):
        k_ms, k_n = kt.get(ph, (0.0, 0))
        avg = k_ms / max(k_n, 1)
        ach = abytes / (avg / 1e3) / 1e9 if avg > 0 else 0.0
        names = PHASE_KERNELS[ph]
        tr = [figs.get(f"{k}.dram_bytes_per_launch") for k in names]
        traffic = sum(tr) if all(t is not None for t in tr) else None
        dp = [figs.get(f"{k}.fp64_ops_per_launch") for k in names]
        dp_ops = sum(dp) if all(t is not None for t in dp) else None
        rl[ph] = {"kernel": PHASE_LABEL[ph], "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                  "frac": ach / hbm_peak, "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                  "algorithmic_bytes_per_launch": abytes, "traffic": traffic,
                  "traffic_source": "ncu capture of this region's launches (same seeded run)" if traffic else None,
                  "ms_avg": avg, "launches_in_window": k_n,
                  "fp64": {"peak_gflops_measured": fp64_peak, "ops_per_launch_ncu": dp_ops,
                           "achieved_gflops": (dp_ops / (avg / 1e3) / 1e9) if (dp_ops and avg > 0) else None,
                           "frac": (dp_ops / (avg / 1e3) / 1e9 / fp64_peak) if (dp_ops and avg > 0) else None}}
    c_ms, c_n = kt.get("collider", (0.0, 0))
    rebuilds = int(s1.nFullRuns - s0.nFullRuns)
    return {
        "value": replica_throughput(world, n, args.steps, ms / 1e3), "ms_per_step": ms / args.steps,
        "steps": args.steps, "warmup": max(args.warmup, 3), "gpu_launches": int(launches),
        "step_graphs": {"mode": GRAPHS, "captures": int(g1[0] - g0[0]), "replays": int(g1[1] - g0[1])},
        "contacts": dict(counts, collider_rebuilds_timed=int(st1.nFullRuns - st0.nFullRuns)),
        "collider": {"window_steps": kw, "rebuilds_in_window": rebuilds,
                     "collider_ms_per_rebuild": (c_ms / c_n) if c_n else None,
                     "steps_per_rebuild": (kw / rebuilds) if rebuilds else None},
        "kernels": {k: {"ms_total": v[0], "launches": v[1], "ms_avg": v[0] / max(v[1], 1)} for k, v in kt.items()},
        "kernels_window_steps": kw, "rooflines": rl, "state": state_tag(args, region, n),
    }


def e2e_measure(h, n, ne, world, local, barrier):
    """End to end through the public C ABI with host buffers, as the engine plug-in runs inside Woo's step
    loop: the kinematic state goes in from pinned host memory once per job (wdem_write_state), then one
    wdem_step call per step (each returns the step's status word to the host: error code and collider
    trigger), then the state comes back to pinned host memory (wdem_read_state).  Beside it, the same with
    the whole kinematic state copied in and out around every single step."""
    import torch
    from woo_gb300 import abi
    pin = {k: torch.empty((n, w_), dtype=torch.float64, pin_memory=True) for k, w_ in
           (("pos", 3), ("vel", 3), ("angVel", 3), ("ori", 4))}
    ptrs = (pin["pos"].data_ptr(), pin["vel"].data_ptr(), pin["angVel"].data_ptr(), pin["ori"].data_ptr())
    h.read_state(n, *ptrs)
    bytes_io = n * (3 + 3 + 3 + 4) * 8
    status_bytes = 128
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h.write_state(n, *ptrs)
    for _ in range(ne):
        h.step(1)
    h.read_state(n, *ptrs)
    torch.cuda.synchronize()
    te = max_over_ranks(time.perf_counter() - t0, world, f"cuda:{local}")
    e2e = {"value": replica_throughput(world, n, ne, te), "unit": "particle-steps/s",
           "h2d_bytes_per_step": bytes_io / ne + ctypes.sizeof(abi.Params),
           "d2h_bytes_per_step": bytes_io / ne + status_bytes, "steps": ne,
           "pattern": "state copied in once and out once per job of `steps` steps (the engine keeps the state "
                      "resident between wdem_step calls), one wdem_step(h, 1) call per step returning its status"}
    nr = min(50, ne)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(nr):
        h.write_state(n, *ptrs)
        h.step(1)
        h.read_state(n, *ptrs)
    torch.cuda.synchronize()
    tr = time.perf_counter() - t0
    roundtrip = {"value": n * nr / tr, "unit": "particle-steps/s", "h2d_bytes_per_step": bytes_io,
                 "d2h_bytes_per_step": bytes_io, "steps": nr,
                 "pattern": "whole kinematic state copied host->device and back around every step"}
    return e2e, roundtrip


def edit_event_cost(h, spec, k=1000):
    """Cost of an outlet / inlet event at the handle's size: k spheres removed on the device
    (wdem_remove_particles) and put back into their slots (wdem_add_particles), against the whole-state
    host round trip that such an event needs without those calls (particles and contacts down, filtered on
    the host, up again).  Wall times of the calls, which synchronise."""
    import torch
    from woo_gb300 import abi
    n = spec.particles.n
    rng = np.random.default_rng(5)
    ids = np.sort(rng.choice(np.arange(6, n), k, replace=False)).astype(np.int32)
    before = h.download_particles(spec.particles.copy())
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    h.remove_particles(ids)
    t_rm = time.perf_counter() - t0
    back = before.take(ids)
    back.vel[:] = 0
    back.angVel[:] = 0
    t0 = time.perf_counter()
    h.add_particles(back, ids)
    t_add = time.perf_counter() - t0
    t0 = time.perf_counter()
    pa = h.download_particles(spec.particles.copy())
    ca = h.download_contacts()
    keep = ~(np.isin(ca.idA, ids) | np.isin(ca.idB, ids))
    ca = ca.take(keep)
    h.upload_particles(pa)
    p = copy_params(spec.params)
    p.step = h.status().step
    h.set_params(p)
    h.upload_contacts(ca)
    t_host = time.perf_counter() - t0
    return {"particles": int(k), "remove_ms": t_rm * 1e3, "add_ms": t_add * 1e3, "host_roundtrip_ms": t_host * 1e3,
            "contacts_in_container": int(ca.n),
            "what": "k spheres removed on the device and re-inserted into their slots, against the host round trip "
                    "of the whole particle and contact state that the same event costs without those calls"}


def common_config(args, spec):
    """The config object both arms print, identical for the same workload so their lines can be compared."""
    return {"workload": args.workload, "n_particles": int(spec.particles.n), "dt": float(spec.params.dt),
            "steps_simulated_before_timing": int(max(args.warmup, 3)), "timed_steps": int(args.steps),
            "l2": "state larger than L2 (no flush needed)"}


def run_gpu(args, rank, world, local):
    import torch
    from woo_gb300 import abi, build as wbuild
    torch.cuda.set_device(local)
    if world > 1 and not torch.distributed.is_initialized():
        torch.distributed.init_process_group("nccl")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    wbuild.build()
    spec = build_scene(args.workload, n=args.n)
    spec.params.arith = {"fma": abi.ARITH_FMA, "dw": abi.ARITH_DW, "exact": abi.ARITH_EXACT}[args.arith]
    n = spec.particles.n
    extra = {}
    if args.workload == "ell200k":
        # train the learned warm start on records of the plain (cold-start) Newton solver, untimed
        p = copy_params(spec.params)
        p.warmStart = abi.WARM_COLD
        hl = new_handle(spec, local, p)
        cap = 5_000_000
        hl.ell_log(cap)
        steps = 0
        while hl.status().ellSolves < cap and steps < 400:
            hl.step(20)
            steps += 20
        R = hl.ell_log_read(cap)
        t0 = time.time()
        losses = hl.warm_train(R, epochs=6, batch=512, lr=3e-3, seed=1)
        w = hl.warm_get_weights()
        hl.close()
        extra["training"] = {"records": int(len(R)), "logged_steps": steps, "epochs": 6, "batch": 512,
                             "loss_first_epoch": float(losses[0]), "loss_last_epoch": float(losses[-1]),
                             "seconds": time.time() - t0}
        extra["variants"] = ell_variants(args, spec, local, world, barrier, w)
        v = extra["variants"]
        extra["warm_start_speedup"] = {
            "contact_pass_vs_newton_cold": v["newton_cold"]["contacts_ms_per_step"] / v["newton_mlp"]["contacts_ms_per_step"],
            "iterations_vs_newton_cold": v["newton_cold"]["iterations_per_solve"] / v["newton_mlp"]["iterations_per_solve"],
            "history_mlp_contact_pass_vs_newton_cold":
                v["newton_cold"]["contacts_ms_per_step"] / v["newton_history_mlp"]["contacts_ms_per_step"],
            "history_mlp_iterations_vs_newton_cold":
                v["newton_cold"]["iterations_per_solve"] / v["newton_history_mlp"]["iterations_per_solve"],
            "history_contact_pass_vs_newton_cold":
                v["newton_cold"]["contacts_ms_per_step"] / v["newton_history"]["contacts_ms_per_step"]}
        h = new_handle(spec, local)
        h.warm_set_weights(w)
    elif args.workload == "batch512":
        # the same scenes one at a time on their own handles (a seeded sample, scaled to all scenes)
        from woo_gb300 import scenes
        nsc = len(spec.info["ranges"])
        rng = np.random.default_rng(11)
        sample = sorted(rng.choice(nsc, min(32, nsc), replace=False).tolist())
        t_total, n_sample = 0.0, 0
        for k in sample:
            single = scenes.single_from_batch(spec, k)
            hs = new_handle(single, local)
            ss = torch.cuda.ExternalStream(hs.stream(), device=local)
            hs.step(max(args.warmup, 3))
            t_total += timed_steps(hs, ss, args.steps, world, local, barrier) / 1e3
            n_sample += single.particles.n
            hs.close()
        scale = nsc / len(sample)
        n_all = spec.particles.n
        extra["scene_by_scene"] = {"sampled_scenes": len(sample), "steps": args.steps,
                                   "seconds_sample": t_total, "seconds_all_estimated": t_total * scale,
                                   "value": n_all * args.steps / (t_total * scale), "unit": "particle-steps/s"}
        h = new_handle(spec, local)
    else:
        h = new_handle(spec, local)
    settled_steps = settle(h, spec) if args.workload == "hertz1M_settled" else 0
    if args.autotune == "on" or (args.autotune == "auto" and args.workload == "batch512"):
        # the fixed default launch shape first, then the autotuner's pick (both untimed for the line;
        # the timed region below runs with the tuned shape)
        st = torch.cuda.ExternalStream(h.stream(), device=local)
        h.step(max(args.warmup, 3))
        ms_fixed = timed_steps(h, st, args.steps, world, local, barrier)
        default_shape = h.launch_shape()
        t0 = time.time()
        tune = h.autotune(5)
        extra["autotune"] = {"default_shape": default_shape, "tuned_shape": tune["shape"],
                             "tuner_ms_per_step_start": tune["ms_start"], "tuner_ms_per_step_best": tune["ms"],
                             "tuning_seconds": time.time() - t0,
                             "gain_tuner": tune["ms_start"] / tune["ms"] if tune["ms"] > 0 else None,
                             "fixed_shape_value_earlier_window": replica_throughput(world, n, args.steps, ms_fixed / 1e3),
                             "how": "coordinate descent over block sizes and blocks per SM of the contact pass, the "
                                    "cull and the integrator, 5 timed steps per candidate (wdem_autotune); gain_tuner is "
                                    "the integrator + contact time per step of the starting shape over the tuned one, "
                                    "measured by the tuner on the same windows of the run"}

    clocks = ClockSampler(local)
    clocks.start()
    main = measure_region(h, spec, args, world, local, barrier, "main")
    e2e, roundtrip = (None, None)
    ne = min(args.e2e_steps, args.steps)
    if ne > 0:
        e2e, roundtrip = e2e_measure(h, n, ne, world, local, barrier)
    if getattr(spec, "cell", None) is not None:
        extra["stress_end_Pa"] = h.stress().tolist()
        extra["packing"] = {"solid_fraction": spec.info.get("phi")}
    h.close()

    settled = None
    if args.workload == "hertz1M" and not args.no_settled:
        # the same spheres settled on the GPU (untimed), then W + K steps with the job's parameters
        hs = new_handle(spec, local)
        t0 = time.time()
        nsettle = settle(hs, spec)
        settle_s = time.time() - t0
        settled = measure_region(hs, spec, args, world, local, barrier, "settled")
        settled["settling"] = {"steps": nsettle, "seconds": settle_s,
                               "how": "damping 0.5: 10 g and 2.5 dt while the cloud falls, 8000 steps at 1 g and 2.5 dt, "
                                      "2000 steps at 1 g and dt"}
        if args.arith == "fma":
            # the same settled run continued with the exact variant (the reference's operations bit for bit)
            pe = copy_params(spec.params)
            pe.arith = abi.ARITH_EXACT
            pe.step = hs.status().step
            hs.set_params(pe)
            ex = measure_region(hs, spec, args, world, local, barrier, "settled_exact")
            settled["exact_arith"] = {k: ex[k] for k in ("value", "ms_per_step", "contacts", "kernels")}
            # and with the contact law in double-word FP32 (the same 1e-12 bar as the contracted variant)
            pd = copy_params(spec.params)
            pd.arith = abi.ARITH_DW
            pd.step = hs.status().step
            hs.set_params(pd)
            dw = measure_region(hs, spec, args, world, local, barrier, "settled_dw")
            settled["dw_arith"] = {k: dw[k] for k in ("value", "ms_per_step", "contacts", "kernels", "rooflines")}
            pf = copy_params(spec.params)
            pf.step = hs.status().step
            hs.set_params(pf)
        if rank == 0 and world == 1 and not args.no_cpu_baseline:
            # the CPU port on this same settled state: particles and contacts (with history) handed over
            pa = hs.download_particles(spec.particles.copy())   # dynamic state over the static arrays
            ca = hs.download_contacts()
            sp = copy_params(spec.params)
            sp.step = hs.status().step
            settled["cpu_baseline"] = cpu_timed(args, sp, pa, ca, None,
                                                f"the same settled {n}-particle state at step {sp.step} "
                                                f"(particles and contacts with history from the GPU), {{steps}} steps after 2 untimed")
            settled["vs_cpu_baseline"] = settled["value"] / settled["cpu_baseline"]["value"]
        settled["edit_events"] = edit_event_cost(hs, spec)
        hs.close()
    clk = clocks.stop()
    clk["interval"] = "sampled over the GPU run: warm-up, timed regions, windows, e2e and settling"

    dominant = max(main["rooflines"], key=lambda k: main["rooflines"][k]["ms_avg"])
    out = {
        "metric": f"{METRIC} ({DESCR[args.workload]})",
        "value": main["value"], "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": main["ms_per_step"], "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded random sequential addition packing)",
        "config": common_config(args, spec),
        "engine": {"parallelism": f"replicas x{world}", "arith": args.arith,
                   "queue_depth": 32 if args.queue_depth is None else args.queue_depth,
                   "step_graphs": main["step_graphs"],
                   "steps_simulated_before_warmup": settled_steps},
        "gpu_launches": main["gpu_launches"],
        "contacts": main["contacts"], "collider": main["collider"],
        "kernels": main["kernels"], "kernels_window_steps": main["kernels_window_steps"],
        "roofline": main["rooflines"][dominant],
        "roofline_other": {k: v for k, v in main["rooflines"].items() if k != dominant},
        "clocks": clk, "e2e": e2e, "e2e_state_roundtrip_every_step": roundtrip,
    }
    if settled is not None:
        out["settled"] = settled
    if "scene_by_scene" in extra:
        extra["batch_speedup_vs_scene_by_scene"] = out["value"] / extra["scene_by_scene"]["value"]
    out.update(extra)
    return out, spec


def cpu_timed(args, params, particles, contacts, cell, sample, max_steps=None):
    """The OpenMP port on the host cores: 2 untimed steps (the initial sort), then timed steps until K steps
    or about --cpu-seconds have run (steady_clock, in the library)."""
    from oracle import bridge
    o = bridge.Oracle(params, particles, contacts=contacts, canonical=False, variant="liborc_omp.so", cell=cell)
    o.set_parallel(True)
    o.step(2)
    steps, total, k = 0, 0.0, 1
    cap = max_steps or args.steps
    while steps < cap and (total < args.cpu_seconds or steps == 0):
        kk = min(k, cap - steps)
        total += o.step_timed(kk)
        steps += kk
        k = min(k * 2, 2000)
    n = particles.n
    return {"value": n * steps / total, "unit": "particle-steps/s", "cores": o.threads(), "kind": "port",
            "steps": steps, "seconds": total,
            "sample": sample.format(steps=steps) + f", OpenMP restatement of Woo's Leapfrog/InsertionSortCollider/"
                                                    f"ContactLoop, {o.threads()} threads"}


def cpu_baseline(args):
    """OpenMP CPU restatement of Woo's step on the host cores.  hertz1M: the same 1M scene and the same
    W warm-up + K timed steps as the GPU arm.  The other workloads: a bounded cut (settled: a cut settled
    on the GPU, its state and contacts handed to the CPU)."""
    from oracle import bridge
    if args.workload == "hertz1M":
        spec = build_scene(args.workload, n=args.n, packer="oracle")
        o = bridge.Oracle(spec.params, spec.particles, canonical=False, variant="liborc_omp.so")
        o.set_parallel(True)
        o.step(max(args.warmup, 3))
        total = o.step_timed(args.steps)
        n = spec.particles.n
        return {"value": n * args.steps / total, "unit": "particle-steps/s", "cores": o.threads(), "kind": "port",
                "steps": args.steps, "seconds": total,
                "sample": f"the same {n}-particle scene and steps: {max(args.warmup, 3)} untimed + {args.steps} timed, "
                          f"OpenMP restatement of Woo's Leapfrog/InsertionSortCollider/ContactLoop, {o.threads()} threads"}, spec
    cuts = {"hertz1M_settled": 100_000, "ell200k": 10_000, "batch512": 16, "peri8M": 10_000, "spheres10k": 10000}
    cut = cuts[args.workload]
    spec = build_scene(args.workload, n=cut, packer="oracle")
    contacts = None
    if args.workload == "hertz1M_settled":
        from woo_gb300 import abi
        h = new_handle(spec, 0)
        settle(h, spec)
        pa = h.download_particles(spec.particles.copy())
        contacts = h.download_contacts()
        spec.params.step = h.status().step
        h.close()
        spec.particles = pa
    if args.workload == "ell200k":
        from woo_gb300 import abi
        spec.params.ellSolver = abi.ELL_BRENT   # the reference's solver
    if args.workload == "batch512":
        # the reference runs independent scenes one by one (a scene per process in its batch system): a
        # seeded sample of the scenes, each on its own, time split evenly
        from woo_gb300 import scenes
        nsc = len(spec.info["ranges"])
        sample = sorted(np.random.default_rng(13).choice(nsc, min(8, nsc), replace=False).tolist())
        psteps, total, threads = 0, 0.0, 1
        for k in sample:
            single = scenes.single_from_batch(spec, k)
            o = bridge.Oracle(single.params, single.particles, canonical=False, variant="liborc_omp.so")
            o.set_parallel(True)
            threads = o.threads()
            o.step(2)
            t, st, kk = 0.0, 0, 10
            while t < args.cpu_seconds / len(sample) and st < 100000:
                t += o.step_timed(kk)
                st += kk
                kk = min(kk * 2, 2000)
            psteps += single.particles.n * st
            total += t
        return {"value": psteps / total, "unit": "particle-steps/s", "cores": threads, "kind": "port",
                "sample": f"{len(sample)} of the scenes (seeded) run one after another, each for ~{args.cpu_seconds / len(sample):.1f} s "
                          f"after 2 untimed steps, OpenMP restatement of Woo's Leapfrog/InsertionSortCollider/ContactLoop, "
                          f"{threads} threads"}, spec
    cb = cpu_timed(args, spec.params, spec.particles, contacts, getattr(spec, "cell", None),
                   f"{args.workload} cut to {spec.particles.n} particles (same density, box scaled), {{steps}} steps after 2 untimed",
                   max_steps=100000)
    return cb, spec


def main():
    global QUEUE_DEPTH, GRAPHS
    args = parse()
    QUEUE_DEPTH = args.queue_depth
    GRAPHS = args.graphs
    rank, world, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return 0
        cb, spec = cpu_baseline(args)
        out = {"metric": f"{METRIC} ({DESCR[args.workload]})",
               "value": cb["value"], "unit": cb["unit"], "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "higher_is_better": True, "impl": "reference", "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic (seeded random sequential addition packing)",
               "config": common_config(args, spec) if args.workload == "hertz1M" else {"workload": args.workload,
                                                                                      "n_particles": int(spec.particles.n)},
               "cpu_baseline": cb,
               "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return 0
    out, spec = run_gpu(args, rank, world, local)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"], _ = cpu_baseline(args)
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
