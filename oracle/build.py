"""Build the CPU oracle (oracle/woo_oracle.cpp) into oracle/_build/liborc.so.

TEST INFRASTRUCTURE: the oracle is what the GPU engine's results are compared with, never part of
the engine.  Compiled with
-ffp-contract=off so that a*b+c stays two IEEE operations on x86-64 and on aarch64 alike.
An OpenMP build (liborc_omp.so) serves as the timed CPU baseline.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
SRC = os.path.join(HERE, "woo_oracle.cpp")


def build(force=False):
    os.makedirs(BUILD, exist_ok=True)
    out = {}
    for name, extra in (("liborc.so", ["-O2"]), ("liborc_omp.so", ["-O3", "-fopenmp"])):
        lib = os.path.join(BUILD, name)
        deps = [SRC, os.path.join(os.path.dirname(HERE), "include", "wdem.h"), __file__]
        if force or not os.path.exists(lib) or any(os.path.getmtime(d) > os.path.getmtime(lib) for d in deps):
            cmd = ["g++", *extra, "-std=c++17", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", SRC, "-o",
                   lib + ".tmp"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"oracle build failed:\n{r.stderr}")
            os.replace(lib + ".tmp", lib)
        out[name] = lib
    return out


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
