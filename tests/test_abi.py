"""The C ABI library loads without a GPU and exports every function include/wdem.h declares; host-only
entry points work on the CPU."""
import ctypes
import os
import re

import numpy as np

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


def test_struct_sizes_match_header():
    # wdem_params: the offsets of the last fields catch any ordering drift
    assert ctypes.sizeof(abi.Material) == 56
    assert abi.Params.materials.offset == ctypes.sizeof(abi.Params) - 8
    assert ctypes.sizeof(abi.Particles) == 8 + 15 * 8


def test_make_cloud_is_seeded_and_non_overlapping(wdem_lib):
    c1, r1 = abi.make_cloud([0, 0, 0], [0.1, 0.1, 0.1], 0.003, 0.006, 400, 5)
    c2, r2 = abi.make_cloud([0, 0, 0], [0.1, 0.1, 0.1], 0.003, 0.006, 400, 5)
    assert np.array_equal(c1, c2) and np.array_equal(r1, r2)
    d = np.linalg.norm(c1[:, None] - c1[None], axis=2)
    np.fill_diagonal(d, np.inf)
    assert (d >= r1[:, None] + r1[None]).all()
    assert (c1 - r1[:, None] >= 0).all() and (c1 + r1[:, None] <= 0.1).all()
    assert abs(np.sum(np.sort(r1)[::-1] - r1)) == 0  # largest first


def test_null_arguments_are_rejected(wdem_lib):
    assert wdem_lib.wdem_create(0, 0, None) == abi.WDEM_ERR_ARG
    assert wdem_lib.wdem_destroy(None) == abi.WDEM_ERR_ARG
    assert wdem_lib.wdem_step(None, 1) == abi.WDEM_ERR_ARG
