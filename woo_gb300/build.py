"""Build libwdem.so (the GB300 DEM engine) in-tree with nvcc for sm_103a.

The library holds the CUDA kernels and the C++ host runtime behind the C ABI of include/wdem.h.
Each translation unit compiles in parallel; FP64 arithmetic is kept IEEE-exact (no FMA contraction
on the device or the host) so that per-contact results reproduce the CPU restatement bit for bit.
The contact and integrator kernels are compiled a second time with WDEM_FMA and FMA contraction (the
contracted variant, selected per handle by wdem_params.arith).
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libwdem.so")

SOURCES = ["k_contact.cu", "k_leapfrog.cu", "k_collider.cu", "wdem_api.cu", "wdem_pack.cu", "k_noalloc.cu", "k_mlp.cu",
           "k_edit.cu"]
# (source, object name, extra flags): the contracted variant of the step kernels
VARIANTS = [("k_contact.cu", "k_contact_fma", ["-DWDEM_FMA", "--fmad=true"]),
            ("k_leapfrog.cu", "k_leapfrog_fma", ["-DWDEM_FMA", "--fmad=true"])]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-Xcompiler", "-O2", "-Xcompiler", "-Wno-deprecated-declarations"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found: the GB300 engine needs the CUDA toolkit to build")
    return exe


def _compile(unit, verbose):
    src, name, extra = unit
    obj = os.path.join(BUILD, name + ".o")
    flags = [f for f in FLAGS if not (extra and f == "--fmad=false")]
    cmd = [nvcc(), *ARCH, *flags, *extra, "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    return obj, (r.stdout + r.stderr)


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, "wdem.h"), __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False):
    """Compile every translation unit and link libwdem.so; returns the library path."""
    if not force and not _stale():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    units = [(s, os.path.splitext(s)[0], []) for s in SOURCES] + VARIANTS
    with ThreadPoolExecutor(max_workers=len(units)) as ex:
        results = list(ex.map(lambda u: _compile(u, verbose), units))
    if verbose:
        for _, log in results:
            sys.stderr.write(log)
    objs = [o for o, _ in results]
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-Xcompiler", "-fPIC", *objs, "-o", tmp, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
