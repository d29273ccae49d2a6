"""Benchmark of the GB300 DEM timestep (particle-steps/s), one JSON line on rank 0.

Workload (default): hertz1M -- 1,000,000 polydisperse HertzMat spheres (r ~ U[2,6] mm, DMT, en=.8,
surfEnergy .01, tanPhi .3/.6) as a loose seeded cloud (solid fraction ~0.3) falling into a
1 x 1 x 2 m walled box, dt = 0.3 x p-wave dt, verletDist 0.1 x rmin, Leapfrog -> collider ->
ContactLoop every step.  A step is one pass of the hot path over all particles; the timed region
covers K consecutive steps of one simulation (state larger than L2 stays resident in HBM).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference] [--workload hertz1M|spheres10k]

--impl reference times the reference algorithm on the host cores (the OpenMP build of the CPU
restatement of Woo's Leapfrog/InsertionSortCollider/ContactLoop), on a bounded cut of the workload.
Multi-GPU: the path does not shard (contacts couple neighbours); N ranks run N independent replicas.
"""
import argparse
import json
import re
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

import numpy as np


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--workload", default="hertz1M", choices=["hertz1M", "spheres10k"])
    ap.add_argument("--e2e-steps", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    return ap.parse_args()


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


def build_scene(name, n=None):
    from woo_gb300 import scenes
    if name == "hertz1M":
        return scenes.hertz1M(n=n or 1_000_000)
    return scenes.spheres10k(n=n or 10000)


def contact_kernel_bytes(cg, shapes, hertz):
    """Algorithmic bytes of one contact-kernel launch: 80 B per particle touched by a contact
    (pos 24, vel 24, angVel 24, radius 8), 288 B per real contact (ids 8, history read 112, history
    write 96, reduction outputs 72), 16 B per potential-only pair (ids 8 + the distance-test data 8);
    Hertz adds 16 B r/w (kn, kt) + 8 B per real contact."""
    live = cg.n
    real = int(cg.real.sum())
    pot = live - real
    touched = len(np.unique(np.concatenate([cg.idA, cg.idB]))) if live else 0
    per_real = 288 + (24 if hertz else 0)
    return 80 * touched + per_real * real + 16 * pot, dict(real=real, potential=pot, touched=touched)


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
    spec = build_scene(args.workload)
    n = spec.particles.n
    h = abi.Handle(n, device=local)
    h.set_params(spec.params)
    h.upload_particles(spec.particles)
    h.set_params(spec.params)
    stream = torch.cuda.ExternalStream(h.stream(), device=local)

    # warm-up (includes the first collider build)
    h.step(max(args.warmup, 3))
    st0 = h.status()
    l0 = h.launch_count()
    hbm_peak, peak_kind = load_peaks()

    h.set_timing(True)
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    ev0.record(stream)
    h.step(args.steps)
    ev1.record(stream)
    ev1.synchronize()
    torch.cuda.synchronize()
    barrier()
    ms = ev0.elapsed_time(ev1)
    clk = clocks.stop()
    launches = h.launch_count() - l0
    kt = h.kernel_times()
    st1 = h.status()
    h.set_timing(False)

    # max over ranks
    t = torch.tensor([ms], device=f"cuda:{local}", dtype=torch.float64)
    if world > 1:
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    ms_max = float(t.item())
    value = world * n * args.steps / (ms_max / 1e3)

    # roofline of the dominant kernel: algorithmic bytes per launch (contact counts at the end of the
    # timed region) over the CUDA-event average launch duration inside the timed region
    cg = h.download_contacts()
    hertz = spec.params.cp2 == abi.CP2_HERTZ
    cbytes, counts = contact_kernel_bytes(cg, spec.particles.shape, hertz)
    lbytes = 256 * n + 80 * counts["real"]   # fused CSR reduction + Leapfrog: 300+52-96 B/particle, 80 B/real contact
    fp64_peak = h.fp64_peak()
    rl = {}
    for kname, label, abytes in (("contacts", "k_contacts (fused Cg2+Cp2+Law2)", cbytes),
                                 ("leapfrog", "k_leapfrog (CSR force gather + Leapfrog + verlet check)", lbytes)):
        k_ms, k_n = kt.get(kname, (0.0, 0))
        avg = k_ms / max(k_n, 1)
        ach = abytes / (avg / 1e3) / 1e9 if avg > 0 else 0.0
        prof = os.path.join(ROOT, "profiles", f"{PROFILE_KERNEL[kname]}_{args.workload}.md")
        traffic = dp_ops = None
        if os.path.exists(prof):
            figs = read_profile_figures(prof)
            traffic = figs.get("dram_bytes_per_launch")
            dp_ops = figs.get("fp64_flops_per_launch")
        rl[kname] = {"kernel": label, "bound": "hbm", "achieved": ach, "peak": hbm_peak, "unit": "GB/s",
                     "frac": ach / hbm_peak, "peak_kind": f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)",
                     "algorithmic_bytes_per_launch": abytes, "traffic": traffic, "ms_avg": avg,
                     "fp64": {"peak_gflops_measured": fp64_peak,
                              "flops_per_launch_ncu": dp_ops,
                              "achieved_gflops": (dp_ops / (avg / 1e3) / 1e9) if (dp_ops and avg > 0) else None,
                              "frac": (dp_ops / (avg / 1e3) / 1e9 / fp64_peak) if (dp_ops and avg > 0) else None}}
    dominant = max(rl, key=lambda k: rl[k]["ms_avg"])

    # end-to-end through the public C ABI with host buffers: per step, the kinematic state goes in from
    # pinned host memory (wdem_write_state), one step runs, and the state comes back (wdem_read_state)
    e2e = None
    ne = min(args.e2e_steps, args.steps)
    if ne > 0:
        pin = {k: torch.empty((n, w), dtype=torch.float64, pin_memory=True) for k, w in
               (("pos", 3), ("vel", 3), ("angVel", 3), ("ori", 4))}
        h.read_state(n, pin["pos"].data_ptr(), pin["vel"].data_ptr(), pin["angVel"].data_ptr(), pin["ori"].data_ptr())
        barrier()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(ne):
            h.write_state(n, pin["pos"].data_ptr(), pin["vel"].data_ptr(), pin["angVel"].data_ptr(), pin["ori"].data_ptr())
            h.step(1)
            h.read_state(n, pin["pos"].data_ptr(), pin["vel"].data_ptr(), pin["angVel"].data_ptr(), pin["ori"].data_ptr())
        e1.record(stream)
        e1.synchronize()
        ems = e0.elapsed_time(e1)
        te = torch.tensor([ems], device=f"cuda:{local}", dtype=torch.float64)
        if world > 1:
            torch.distributed.all_reduce(te, op=torch.distributed.ReduceOp.MAX)
        bytes_io = n * (3 + 3 + 3 + 4) * 8
        e2e = {"value": world * n * ne / (float(te.item()) / 1e3), "unit": "particle-steps/s",
               "h2d_bytes_per_step": bytes_io, "d2h_bytes_per_step": bytes_io, "steps": ne}

    out = {
        "metric": "particle-steps/s per GB300 (plain DEM step, HertzDMT settling)" if args.workload == "hertz1M"
        else "particle-steps/s per GB300 (plain DEM step, FrictMat IdealElPl)",
        "value": value, "unit": "particle-steps/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded random sequential addition cloud)",
        "config": {"workload": args.workload, "n_particles": n, "dt": spec.params.dt,
                   "parallelism": f"replicas x{world}", "l2": "state larger than L2 (no flush needed)",
                   "steps_simulated_before_timing": int(max(args.warmup, 3))},
        "gpu_launches": int(launches),
        "kernels": {k: {"ms_total": v[0], "launches": v[1], "ms_avg": v[0] / max(v[1], 1)} for k, v in kt.items()},
        "contacts": dict(counts, collider_rebuilds_timed=int(st1.nFullRuns - st0.nFullRuns)),
        "roofline": rl[dominant],
        "roofline_other": {k: v for k, v in rl.items() if k != dominant},
        "clocks": clk,
        "e2e": e2e,
    }
    h.close()
    return out, spec


def cpu_baseline(args, full_n):
    """OpenMP CPU restatement of Woo's step on the host cores, on a bounded cut of the workload."""
    from oracle import bridge
    cut = 100_000 if args.workload == "hertz1M" else 10000
    spec = build_scene(args.workload, n=cut)
    o = bridge.Oracle(spec.params, spec.particles, canonical=False, variant="liborc_omp.so")
    o.set_parallel(True)
    o.step(2)  # initial sort + first contacts, not timed
    steps, total = 0, 0.0
    k = 10
    while total < args.cpu_seconds and steps < 100000:
        total += o.step_timed(k)
        steps += k
        k = min(k * 2, 2000)
    n = spec.particles.n
    return {"value": n * steps / total, "unit": "particle-steps/s", "cores": o.threads(), "kind": "port",
            "sample": f"{args.workload} cut to {n} particles (same density, box scaled), {steps} steps after 2 untimed, "
                      f"OpenMP restatement of Woo's Leapfrog/InsertionSortCollider/ContactLoop, {o.threads()} threads"}


PROFILE_KERNEL = {"leapfrog": "k_leapfrog", "contacts": "k_contacts"}


def read_profile_figures(path):
    """`- name: number` lines of an ncu summary under profiles/ (per-launch figures of one capture)."""
    figs = {}
    with open(path) as f:
        for line in f:
            m = re.match(r"^- (\w+): ([0-9.eE+-]+)\s*$", line)
            if m:
                figs[m.group(1)] = float(m.group(2))
    return figs


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        if rank != 0:
            return 0
        cb = cpu_baseline(args, None)
        out = {"metric": "particle-steps/s per GB300 (plain DEM step, HertzDMT settling)" if args.workload == "hertz1M"
               else "particle-steps/s per GB300 (plain DEM step, FrictMat IdealElPl)",
               "value": cb["value"], "unit": cb["unit"], "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
               "higher_is_better": True, "impl": "reference", "scaling": "weak", "vs_baseline": None, "dtype": "f64",
               "data": "synthetic", "config": {"workload": args.workload},
               "cpu_baseline": cb,
               "e2e": {"value": cb["value"], "unit": cb["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return 0
    out, spec = run_gpu(args, rank, world, local)
    if rank == 0:
        if world == 1 and not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(args, spec.particles.n)
        print(json.dumps(out))
    return 0


if __name__ == "__main__":
    sys.exit(main())
