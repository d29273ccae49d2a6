"""The double-word arithmetic of the contact law (woo_gb300/csrc/wdem_dw.cuh) on the CPU: the header compiles
for the host, and a seeded harness measures each operation against long double on magnitudes 1e-12 to
1e12 (the contact law's range; products stay far above FP32's subnormals).  The bounds, in u^2 = 2^-48
(u = 2^-24), are those Joldes, Muller and Popescu prove for the algorithms: addition 3, addition of a
float 2, multiplication 5, multiplication by a float 2, division 15; the square root (one Newton step
with an exact square) is held to 4.  Conversions from double lose at most one u^2 (the high word is
exact, the low word rounded) and keep the words normalised; conversions back to double are exact."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_dw_error_bounds(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    exe = str(tmp_path / "dw_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-o", exe, os.path.join(HERE, "native", "dw_check.cpp")],
                   check=True, capture_output=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    r = {k: float(v) for k, v in (line.split() for line in out.strip().splitlines())}
    assert r["from"] <= 1.01
    assert r["add"] <= 3.0
    assert r["addF"] <= 2.0
    assert r["mul"] <= 5.0
    assert r["mulF"] <= 2.0
    assert r["div"] <= 15.0
    assert r["sqrt"] <= 4.0
    assert r["unnormalised"] == 0
    assert r["roundtrip"] == 0
