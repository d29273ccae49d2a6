"""Ellipsoids in the oracle: the reference's known answers (py/tests/test_ellipsoid.py) and checks of
the Perram-Wertheim solve, the wall functor and the aspherical Leapfrog."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes


def test_mass_inertia():
    """py/tests/test_ellipsoid.py:64-72: m = rho 4/3 pi abc, I = m/5 (b^2+c^2, a^2+c^2, a^2+b^2)."""
    m, inertia = scenes.ellipsoid_mass_inertia([[1.0, 2.0, 3.0]], 1.0)
    mm = (4 / 3.0) * math.pi * 6
    assert m[0] == pytest.approx(mm, rel=1e-15)
    assert np.allclose(inertia[0], mm / 5 * np.array([13.0, 10.0, 5.0]), rtol=1e-15)


def _two_ellipsoids(scale, solver):
    """The scene of py/tests/test_ellipsoid.py:24-57: two fixed ellipsoids touching externally along
    their common local x axis, the whole setup rotated by gOri; #1 moves towards #0 at 0.1 m/s, dt 0.1."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1e3, young=1e8, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    g = scenes.quat_from_axis_angle((0.1, 1, 0.3), math.pi / 3.0)
    g = g / np.linalg.norm(g)
    centers = np.array([[0.0, 0, 0], scenes.quat_rotate(g, scale * np.array([0.3, 0, 0]))])
    semi = scale * np.array([[0.1, 0.2, 0.1], [0.2, 0.1, 0.1]])
    pa = scenes.assemble_ellipsoids(centers, semi, np.array([g, g]), 0, [], mats_py)
    pa.flags[:] = abi.DOF_ALL
    pa.vel[1] = scenes.quat_rotate(g, np.array([-0.1, 0, 0]))
    p = scenes.default_params(mats, dt=0.1, damping=0.4, verletDist=0.0, noBreak=1, ellSolver=solver)
    return p, pa


@pytest.mark.parametrize("solver", [abi.ELL_BRENT, abi.ELL_NEWTON])
@pytest.mark.parametrize("scale", [0.5 / 3.0, 1.0 / 3.0, 10.0 / 3.0, 100.0 / 3.0, 1000 / 3.0])
def test_normal_displacement_ellipsoid(scale, solver):
    """py/tests/test_ellipsoid.py:24-57: after one step the overlap is the 0.01 m the second ellipsoid
    moved, within 1e-5 x 0.01, at every scale."""
    p, pa = _two_ellipsoids(scale, solver)
    o = bridge.Oracle(p, pa)
    o.step(1)
    c = o.contacts()
    assert c.n == 1 and c.real[0] == 1
    assert c.uN[0] == pytest.approx(-0.01, abs=1e-5 * 0.01)


def test_wall_ellipsoid():
    """Cg2_Wall_Ellipsoid_L6Geom: the overlap is the extent along the wall axis minus the distance of
    the centre, and the contact point lies in the wall plane."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1e3, young=1e8, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    q = scenes.quat_from_axis_angle((1, 2, 3), math.pi / 4.0)
    semi = np.array([[0.3, 0.2, 0.1]])
    # extent along z: norm of row z of [q*(a e_x), q*(b e_y), q*(c e_z)]
    cols = np.stack([scenes.quat_rotate(q, semi[0, k] * np.eye(3)[k]) for k in range(3)], axis=1)
    ext = math.sqrt(float(cols[2] @ cols[2]))
    pa = scenes.assemble_ellipsoids(np.array([[0.0, 0.0, ext - 0.001]]), semi, q[None, :], 0,
                                    [(2, 1, 0.0, 0)], mats_py)
    pa.flags[:] = abi.DOF_ALL
    p = scenes.default_params(mats, dt=1e-6, damping=0.0, verletDist=0.0)
    o = bridge.Oracle(p, pa)
    o.step(1)
    c = o.contacts()
    assert c.n == 1 and c.real[0] == 1 and c.idA[0] == 0
    assert c.uN[0] == pytest.approx(-0.001, abs=1e-15)
    assert c.contPt[0, 2] == 0.0
    assert np.allclose(c.trsf[0][:3], [0, 0, 1])


@pytest.mark.parametrize("solver", [abi.ELL_BRENT, abi.ELL_NEWTON])
def test_spheres_through_perram_wertheim(solver):
    """Two spheres given as ellipsoids with equal semi-axes: uN = |R| - r1 - r2 (the sphere functor's
    answer) and the contact point where the spheres scaled by the same factor touch, |R| r1 / (r1 + r2)
    along the centre line, within the solver's accuracy."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1e3, young=1e8, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    rng = np.random.default_rng(1)
    for _ in range(5):
        r1, r2 = rng.uniform(0.5, 2.0, 2)
        d = rng.normal(size=3)
        d /= np.linalg.norm(d)
        dist = (r1 + r2) * 0.97
        semi = np.array([[r1, r1, r1], [r2, r2, r2]])
        oris = scenes.random_quaternions(2, rng)
        pa = scenes.assemble_ellipsoids(np.array([[0.0, 0, 0], dist * d]), semi, oris, 0, [], mats_py)
        pa.flags[:] = abi.DOF_ALL
        p = scenes.default_params(mats, dt=1e-9, damping=0.0, verletDist=0.0, ellSolver=solver)
        o = bridge.Oracle(p, pa)
        o.step(1)
        c = o.contacts()
        tol = 1e-6 if solver == abi.ELL_BRENT else 1e-12
        assert c.uN[0] == pytest.approx(dist - r1 - r2, abs=tol * (r1 + r2))
        cp = dist * r1 / (r1 + r2) * d
        assert np.allclose(c.contPt[0], cp, atol=tol * (r1 + r2) * 10)


def test_brent_agrees_with_exact_maximiser():
    """Brent at the reference's 32 (capped to 26) bits finds lambda to ~3e-8 and the contact function
    value to double precision: forces of a settling ellipsoid cloud after one step agree with the
    exact maximiser within 1e-6 relative."""
    out = {}
    for solver in (abi.ELL_BRENT, abi.ELL_NEWTON):
        spec = scenes.ellipsoid_cloud(300, 4, dense=0.7, ellSolver=solver)
        o = bridge.Oracle(spec.params, spec.particles)
        o.step(1)
        out[solver] = (o.contacts(), o.particles(), o.ell_stats())
    cb, pb, sb = out[abi.ELL_BRENT]
    cn, pn, sn = out[abi.ELL_NEWTON]
    assert cb.n == cn.n and np.array_equal(cb.keys(), cn.keys())
    r = cb.real.astype(bool)
    assert r.sum() > 20
    scale = np.abs(cn.force[r]).max()
    assert np.allclose(cb.force[r], cn.force[r], rtol=0, atol=1e-6 * scale)
    assert sb[0] > 0 and sb[1] / sb[0] > 5      # Brent: several evaluations per solve


def test_free_rotation_conserves_angular_momentum():
    """Aspherical Leapfrog without torque: DemData.angMom is constant and the orientation stays unit."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1e3, young=1e8, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    q = scenes.quat_from_axis_angle((0.3, -1, 0.2), 0.7)
    pa = scenes.assemble_ellipsoids(np.zeros((1, 3)), np.array([[0.3, 0.2, 0.1]]), q[None, :], 0, [], mats_py)
    pa.angVel[0] = [3.0, -1.0, 2.0]
    p = scenes.default_params(mats, dt=1e-4, damping=0.0, verletDist=0.0)
    o = bridge.Oracle(p, pa)
    o.step(1)
    l0 = o.particles().angMom[0].copy()
    o.step(500)
    pp = o.particles()
    assert np.array_equal(pp.angMom[0], l0)
    assert abs(np.linalg.norm(pp.ori[0]) - 1) < 1e-15
    assert np.linalg.norm(pp.angVel[0]) > 0
