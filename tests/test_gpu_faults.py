"""Failure handling of the GPU engine, exercised from the host (no kernel is made to fault or hang):

- the periodic double contact (boxes overlapping across two periods) comes back from the step as
  WDEM_ERR_TOO_BIG with a message, as the reference's collider throws (py/tests/test_pbc.py:145-155,
  InsertionSortCollider.cpp:286-290), while a sphere spanning more than half the cell without a double
  contact is not an error (test_pbc.py:130-144);
- a contact container beyond the caller's limit (wdem_set_contact_limit) comes back as WDEM_ERR_OVERFLOW
  before anything is allocated, and the device stays usable;
- a container that outgrows its initial capacity many times over regrows and keeps bit-exact parity.
Every failing call returns within its own bounded work; the test then runs a fresh handle on the same
device to show the context is intact."""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def _two_spheres(c0, r0, c1, r1):
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    pa = scenes.assemble(np.array([c0, c1], float), np.array([r0, r1]), 0, [], mats_py)
    p = scenes.default_params(mats, dt=1e-8, gravity=(0, 0, 0), damping=0.0)
    return scenes.SceneSpec(p, mats, pa, "two", cell=dict(hSize=np.eye(3), trsf=np.eye(3), gradV=np.zeros((3, 3)),
                                                          nextGradV=np.zeros((3, 3))))


def _fresh_handle_works():
    spec = scenes.random_cloud(300, 2, dense=0.9)
    h = gpu_handle(spec)
    h.step(20)
    assert h.status().nReal >= 0
    h.close()


def test_periodic_double_contact_is_an_error(wdem_lib):
    spec = _two_spheres((.3, .5, .5), .4, (.8, .9, .5), .2)
    h = gpu_handle(spec)
    with pytest.raises(abi.WdemError, match="ambiguous periodic contact") as ei:
        h.step(1)
    assert ei.value.code == abi.WDEM_ERR_TOO_BIG
    h.close()
    _fresh_handle_works()


@pytest.mark.parametrize("shift", [(0, 0, 0), (13, 14, 15)])
def test_periodic_over_half_cell_contact(wdem_lib, shift):
    spec = _two_spheres(np.array([.3, .5, .5]) + shift, .4, (.7, .9, .5), .1)
    h = gpu_handle(spec)
    h.step(1)
    c = h.download_contacts()
    assert c.n == 1 and (c.idA[0], c.idB[0]) == (0, 1)
    assert tuple(c.cellDist[0]) == shift
    h.close()


def test_contact_limit_overflow(wdem_lib):
    spec = scenes.random_cloud(3000, 3, box=(0.15, 0.15, 0.15), dense=0.8)
    h = gpu_handle(spec)
    h.set_contact_limit(100)
    with pytest.raises(abi.WdemError, match="exceed the limit") as ei:
        h.step(1)
    assert ei.value.code == abi.WDEM_ERR_OVERFLOW
    h.close()
    # the same scene within a limit that suffices runs as the oracle does
    h = gpu_handle(spec)
    h.set_contact_limit(10_000_000)
    o = bridge.Oracle(spec.params, spec.particles)
    h.step(10)
    o.step(10)
    assert_same_particles(gpu_particles(h, spec.particles.n), o.particles())
    h.close()
    _fresh_handle_works()


def test_contact_buffer_regrows(wdem_lib):
    """The first collider run finds tens of times the initial container capacity (1024 pairs); the
    buffers regrow in place and the run stays bit-exact against the oracle."""
    spec = scenes.random_cloud(6000, 12, box=(0.2, 0.2, 0.2), rmin=0.003, rmax=0.005, dense=0.75)
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    for k in (1, 30):
        h.step(k)
        o.step(k)
    cg = h.download_contacts()
    assert cg.n > 20 * 1024
    assert_same_particles(gpu_particles(h, spec.particles.n), o.particles())
    assert_same_contacts(cg, o.contacts())
    h.close()
