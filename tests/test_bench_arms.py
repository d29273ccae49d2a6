"""bench.py's CPU arm (--impl reference) on a small cut: it prints the JSON line with the same config keys as
the GPU arm and never loads the engine library (the timed CPU code is the oracle's OpenMP build only)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SCRIPT = r"""
import io, contextlib, json, runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--n", "8000", "--steps", "4", "--warmup", "3", "--cpu-seconds", "2"]
buf = io.StringIO()
with contextlib.redirect_stdout(buf):
    try:
        runpy.run_path(sys.argv_path, run_name="__main__")
    except SystemExit:
        pass
maps = open("/proc/self/maps").read()
print(json.dumps({"line": buf.getvalue().strip().splitlines()[-1], "libwdem": "libwdem" in maps,
                  "liborc_omp": "liborc_omp" in maps}))
"""


def test_reference_arm_uses_oracle_only():
    code = "import sys; sys.argv_path = %r\n" % os.path.join(ROOT, "bench.py") + SCRIPT
    r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert not res["libwdem"], "the CPU arm loaded the engine library"
    assert res["liborc_omp"]
    line = json.loads(res["line"])
    assert line["impl"] == "reference" and line["value"] > 0
    cfg = line["config"]
    assert cfg["workload"] == "hertz1M" and cfg["timed_steps"] == 4 and cfg["steps_simulated_before_timing"] == 3
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0


def _bench_module():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_profile_traffic_figures_cover_the_phases():
    """The line's roofline `traffic` comes from the ncu summaries under profiles/ that record the same
    state: the default run's states (1M spheres, 5 warm-up and 20 timed steps; the free-falling window and
    the settled one, contracted and double-word) each find DRAM bytes per launch for every kernel of both
    phases, and the tag the bench computes for the defaults is the one those summaries record."""
    import argparse
    bench = _bench_module()
    steps = bench.DEFAULT_STEPS["hertz1M"]
    old = sys.argv
    try:
        sys.argv = ["bench.py"]
        args = bench.parse()
    finally:
        sys.argv = old
    ns = argparse.Namespace(workload=args.workload, warmup=args.warmup, steps=steps, arith=args.arith)
    n = 1_000_006
    tags = [bench.state_tag(ns, "main", n), bench.state_tag(ns, "settled", n)]
    assert tags[0] == "hertz1M/main/n=1000006/warmup=5/steps=20"
    ns.arith = "dw"
    tags.append(bench.state_tag(ns, "settled", n))
    assert tags[2].endswith("/arith=dw")
    for tag in tags:
        figs = bench.read_profile_figures(tag)
        for kernels in bench.PHASE_KERNELS.values():
            for k in kernels:
                assert figs.get(f"{k}.dram_bytes_per_launch", 0) > 0, (tag, k)
