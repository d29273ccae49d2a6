"""wdem_get_stress_noalloc (stress with its scratch in a fixed device array) against wdem_get_stress.

The two sum the same per-contact terms in a different order, so they agree to rounding: relative
1e-12 of the largest component.  Two calls in a row give identical results (the completion counter
is cleared by each call; nothing else carries over).  The file is named to be collected last, so the
shared device array has been through whatever the other GPU tests left behind."""
import numpy as np
import pytest

from woo_gb300 import scenes

from helpers import gpu_handle

pytestmark = pytest.mark.gpu

TOL = 1e-12


def _compare(h):
    ref = h.stress()
    a = h.stress_noalloc()
    b = h.stress_noalloc()
    scale = np.abs(ref).max()
    assert scale > 0
    assert np.array_equal(a, b), "two calls in a row differ"
    assert np.allclose(a, ref, rtol=0, atol=TOL * scale), f"{a} vs {ref}"
    return a


@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_noalloc_stress_periodic(wdem_lib, law):
    spec = scenes.periodic_cloud(500, 3, law=law, shear=0.2)
    h = gpu_handle(spec)
    h.step(50)
    _compare(h)
    h.step(25)
    _compare(h)


def test_noalloc_stress_walls(wdem_lib):
    spec = scenes.random_cloud(1500, 4, dense=0.85)
    h = gpu_handle(spec)
    h.step(40)
    _compare(h)


def test_noalloc_stress_many_blocks(wdem_lib):
    """More contacts than one block's chunk (4096): several partial sums and the last-block total."""
    spec = scenes.random_cloud(6000, 9, box=(0.2, 0.2, 0.2), dense=0.85, walls=False, gravity=(0, 0, 0))
    h = gpu_handle(spec)
    h.step(5)
    assert h.contact_count() > 3 * 4096
    _compare(h)


def test_noalloc_stress_allocates_nothing(wdem_lib):
    """On a fresh handle, before any call of the allocating wdem_get_stress: the first call looks up the
    scratch array's address (and may load the module), the second call must leave the device's free
    memory exactly as it was."""
    torch = pytest.importorskip("torch")
    spec = scenes.random_cloud(1500, 6, dense=0.85)
    h = gpu_handle(spec)
    h.step(40)
    a = h.stress_noalloc()
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(0)
    b = h.stress_noalloc()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(0)
    assert free1 == free0, f"free device memory changed by {free0 - free1} bytes"
    assert np.array_equal(a, b)
    ref = h.stress()
    assert np.allclose(a, ref, rtol=0, atol=TOL * np.abs(ref).max())


def test_noalloc_stress_no_contacts(wdem_lib):
    spec = scenes.random_cloud(20, 1, box=(1.0, 1.0, 1.0), walls=False, gravity=(0, 0, 0))
    h = gpu_handle(spec)
    h.step(1)
    assert np.array_equal(h.stress_noalloc(), np.zeros((3, 3)))
