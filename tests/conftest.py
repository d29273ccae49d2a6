import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libwdem.so")
    config.addinivalue_line("markers", "host_engines: scripts with outlets/inlets (host engines between GPU steps)")


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


HAS_GPU = _has_gpu()


def _order(item):
    # the kernel parity tests first, then the scripts with host engines (outlets, inlets), so that a
    # failure there under -x does not hide the kernel results; test_zz_* stay last
    mod = getattr(item, "module", None)
    if mod is not None and mod.__name__.startswith("test_zz"):
        return 2
    return 1 if "host_engines" in item.keywords else 0


def pytest_collection_modifyitems(config, items):
    items.sort(key=_order)
    if HAS_GPU:
        return
    skip = pytest.mark.skip(reason="no CUDA device")
    for it in items:
        if "gpu" in it.keywords:
            it.add_marker(skip)


@pytest.fixture(scope="session")
def wdem_lib():
    from woo_gb300 import build, abi
    build.build()
    return abi.load()
