"""Periodic cell on the GPU against the oracle: Leapfrog's gradV2 integration, the periodic pair set
with Contact.cellDist (spatialOverlapPeri), contact geometry and velocity at the shifted image
(Cell.intrShiftPos / intrShiftVel), energy with the step-0 rule, and the stress tensor.  Same
bar as the aperiodic parity: bitwise except sin/cos-driven orientations."""
import ctypes
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def _check_same(h, o, n):
    assert_same_particles(gpu_particles(h, n), o.particles())
    cg, co = h.download_contacts(), o.contacts()
    assert_same_contacts(cg, co)
    assert np.array_equal(cg.cellDist, co.cellDist), "cellDist differs"
    return cg


@pytest.mark.parametrize("law", ["frict", "hertz"])
@pytest.mark.parametrize("shear", [0.0, 0.25])
def test_periodic_multistep_bitexact(wdem_lib, law, shear):
    spec = scenes.periodic_cloud(500, 7, law=law, shear=shear)
    n = spec.particles.n
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles, cell=spec.cell)
    crossing = 0
    for chunk in (1, 9, 90, 200):
        h.step(chunk)
        o.step(chunk)
        cg = _check_same(h, o, n)
        crossing = max(crossing, int(np.count_nonzero(np.any(cg.cellDist != 0, axis=1) & (cg.real == 1))))
    assert crossing > 0, "no real contact across the periodic boundary"
    assert h.status().nFullRuns == o.n_full_runs()
    cg_cell, co_cell = h.cell(), o.cell()
    for k in ("hSize", "trsf", "gradV", "pprevHsize"):
        assert np.array_equal(cg_cell[k], co_cell[k]), k


def test_periodic_stress(wdem_lib):
    spec = scenes.periodic_cloud(500, 11, law="hertz", shear=0.1)
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles, cell=spec.cell)
    h.step(60)
    o.step(60)
    sg, so = h.stress(), o.stress()
    assert np.abs(so).max() > 0
    # the sum runs in a different order on the two sides: relative 1e-12 of the largest component
    assert np.allclose(sg, so, rtol=0, atol=1e-12 * np.abs(so).max())


def test_periodic_energy(wdem_lib):
    """EnergyTracker over a periodic run with nextGradV != 0: no Leapfrog energy in step 0
    (Leapfrog.cpp:132), fluctuation velocities for the kinetic energy afterwards."""
    spec = scenes.periodic_cloud(400, 5, law="frict", shear=0.1, damping=0.2)
    spec.params.trackEnergy = 1
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles, cell=spec.cell)
    h.step(1); o.step(1)
    eg, eo = h.energy(), o.energy()
    assert eo["kinetic"] == 0.0 and eg["kinetic"] == 0.0
    h.step(80); o.step(80)
    eg, eo = h.energy(), o.energy()
    for k in eo:
        assert eg[k] == pytest.approx(eo[k], rel=1e-12, abs=1e-15), k
    assert eo["kinetic"] > 0


def test_periodic_incident_velocity(wdem_lib):
    """py/tests/test_pbc.py:86-95 on the GPU: sphere ten cells away along z, nextGradV = diag(0,0,-1);
    the incident velocity of the contact, corrected by Cell.intrShiftVel, is the initial 5 m/s."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7, ktDivKn=0.2, tanPhi=math.tan(0.5))]
    mats = scenes.materials_array(mats_py)
    pa = scenes.assemble(np.array([[1.0, 1, 1], [1.0, 2.0, 31.0]]), np.array([0.5, 0.5]), 0, [], mats_py,
                         vel=np.array([[0, 0, 0], [0, 0, 5.0]]))
    p = scenes.default_params(mats, dt=0.0, damping=0.0, noBreak=1)
    spec = scenes.SceneSpec(p, mats, pa, cell=dict(hSize=np.diag([2.5, 2.5, 3.0]), nextGradV=np.diag([0, 0, -1.0])))
    h = gpu_handle(spec)
    h.step(1)
    v = gpu_particles(h, 2).vel
    assert v[1, 2] == pytest.approx(5.0 - 31.0) and v[0, 2] == pytest.approx(-1.0)
    p.dt = 1e-10
    p.step = 1
    h.set_params(p)
    h.step(1)
    c = h.download_contacts()
    assert c.n == 1 and c.real[0] == 1
    assert np.array_equal(c.cellDist[0], [0, 0, -10])
    assert np.linalg.norm(c.geomVel[0]) == pytest.approx(5.0, abs=1e-7)


def test_periodic_rejects_walls(wdem_lib):
    spec = scenes.random_cloud(50, 1)
    h = gpu_handle(spec)
    with pytest.raises(abi.WdemError):
        h.set_cell(np.eye(3))


@pytest.mark.parametrize("damping", [0.0, 0.3])
def test_periodic_damped_changing_gradient(wdem_lib, damping):
    """Damping on the fluctuation velocity and spin, and a velocity gradient that changes between
    steps (L+ != L-, non-zero deltaSpinVec): bitwise against the oracle."""
    spec = scenes.periodic_cloud(400, 11, law="frict", shear=0.1, rate=3.0, damping=damping)
    n = spec.particles.n
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles, cell=spec.cell)
    rng = np.random.default_rng(2)
    for chunk in (1, 20, 40, 100):
        h.step(chunk)
        o.step(chunk)
        _check_same(h, o, n)
        g = rng.normal(0, 2.0, (3, 3))
        c = o.cell()
        h.set_cell(c["hSize"], c["trsf"], c["gradV"], g)
        o.set_cell(c["hSize"], c["trsf"], c["gradV"], g)
    assert np.array_equal(h.cell()["hSize"], o.cell()["hSize"])


def test_densified_periodic_packing(wdem_lib):
    """Radius-growth densification of a loose periodic packing on the GPU: the target solid fraction,
    the original radii, real contacts, and then the sheared dense packing bitwise against the oracle."""
    loose = scenes.peri_shear(n=3000, seed=3)
    spec = scenes.densify_periodic(loose, phi_target=0.62, stages=8, steps_per_stage=100, relax=200)
    assert spec.info["phi"] == pytest.approx(0.62, rel=1e-9)
    assert np.array_equal(spec.particles.radius, loose.particles.radius)
    n = spec.particles.n
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles, cell=spec.cell)
    for chunk in (1, 30, 120):
        h.step(chunk)
        o.step(chunk)
        cg = _check_same(h, o, n)
    assert int(cg.real.sum()) > n
