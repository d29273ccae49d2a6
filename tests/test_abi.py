"""The C ABI library loads without a GPU and exports every function include/wdem.h declares; host-only
entry points work on the CPU."""
import ctypes
import subprocess
import os
import re

import numpy as np
import pytest

from woo_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    src = open(os.path.join(ROOT, "include", "wdem.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*)\s+(wdem_\w+)\s*\(", src, re.M)))


def test_exports_every_declared_function(wdem_lib):
    names = declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(wdem_lib, n), n
    assert set(names) == set(abi.EXPORTS)


def test_abi_version(wdem_lib):
    assert wdem_lib.wdem_abi_version() == abi.ABI_VERSION


def test_struct_layouts_match_header(tmp_path):
    """Every field offset and struct size of the ctypes mirrors equals what the C compiler makes of
    include/wdem.h."""
    structs = {"wdem_material": abi.Material, "wdem_params": abi.Params, "wdem_particles": abi.Particles,
               "wdem_contacts": abi.Contacts, "wdem_cell": abi.Cell, "wdem_status": abi.Status,
               "wdem_launch_shape": abi.LaunchShape}
    lines = ['#include <stdio.h>', '#include <stddef.h>', f'#include "{ROOT}/include/wdem.h"', "int main(void) {"]
    for cname, cls in structs.items():
        lines.append(f'  printf("{cname} size %zu\\n", sizeof({cname}));')
        for fname, _ in cls._fields_:
            lines.append(f'  printf("{cname} {fname} %zu\\n", offsetof({cname}, {fname}));')
    lines.append("  return 0; }")
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c11", "-o", str(exe), str(src)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, cls in structs.items():
        assert got[(cname, "size")] == ctypes.sizeof(cls), cname
        for fname, _ in cls._fields_:
            assert got[(cname, fname)] == getattr(cls, fname).offset, f"{cname}.{fname}"


def test_make_cloud_is_seeded_and_non_overlapping(wdem_lib):
    c1, r1 = abi.make_cloud([0, 0, 0], [0.1, 0.1, 0.1], 0.003, 0.006, 400, 5)
    c2, r2 = abi.make_cloud([0, 0, 0], [0.1, 0.1, 0.1], 0.003, 0.006, 400, 5)
    assert np.array_equal(c1, c2) and np.array_equal(r1, r2)
    d = np.linalg.norm(c1[:, None] - c1[None], axis=2)
    np.fill_diagonal(d, np.inf)
    assert (d >= r1[:, None] + r1[None]).all()
    assert (c1 - r1[:, None] >= 0).all() and (c1 + r1[:, None] <= 0.1).all()
    assert abs(np.sum(np.sort(r1)[::-1] - r1)) == 0  # largest first


@pytest.mark.parametrize("periodic", [False, True])
def test_make_cloud_radii_non_overlapping(wdem_lib, periodic):
    """Random sequential addition of given radii: seeded, no overlap (under the minimum image when periodic),
    inside the box (centres only, when periodic)."""
    rng = np.random.default_rng(3)
    rin = np.sort(rng.uniform(0.02, 0.05, 300))[::-1]
    L = 1.0
    c1, r1 = abi.make_cloud_radii([0, 0, 0], [L, L, L], rin, 9, periodic=periodic)
    c2, r2 = abi.make_cloud_radii([0, 0, 0], [L, L, L], rin, 9, periodic=periodic)
    assert np.array_equal(c1, c2) and np.array_equal(r1, r2)
    assert len(r1) > 200
    dv = c1[:, None] - c1[None]
    if periodic:
        dv -= L * np.round(dv / L)
        assert (c1 >= 0).all() and (c1 < L).all()
    else:
        assert (c1 - r1[:, None] >= 0).all() and (c1 + r1[:, None] <= L).all()
    d = np.linalg.norm(dv, axis=2)
    np.fill_diagonal(d, np.inf)
    assert (d >= r1[:, None] + r1[None]).all()


def test_null_arguments_are_rejected(wdem_lib):
    assert wdem_lib.wdem_create(0, 0, None) == abi.WDEM_ERR_ARG
    assert wdem_lib.wdem_destroy(None) == abi.WDEM_ERR_ARG
    assert wdem_lib.wdem_step(None, 1) == abi.WDEM_ERR_ARG
