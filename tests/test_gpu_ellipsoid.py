"""Ellipsoids on the GPU against the oracle.

With the reference's solver (Brent, WDEM_ELL_BRENT) the GPU runs the same IEEE operations as the
oracle, so the state is compared bit for bit (sin/cos-driven sphere orientations to 1e-12).  The
Newton solver (WDEM_ELL_NEWTON, converged to |d lambda| <= 1e-10) is compared with the oracle's
exact maximiser (bisection on dS/dlambda to the last bit) within 1e-9 relative on forces."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def _mixed_cloud(seed, solver, **kw):
    """Ellipsoids (semi-axes a, .7a, .5a) and 20 % spheres in a walled box, overlapping at the start."""
    spec = scenes.ellipsoid_cloud(300, seed, dense=0.72, ellSolver=solver, sphere_frac=0.2, **kw)
    return spec


def _particles_with_angmom(h, n):
    pa = abi.ParticleArrays(n)
    return h.download_particles(pa)


@pytest.mark.parametrize("seed", [1, 2])
def test_brent_multistep_bitexact(wdem_lib, seed):
    spec = _mixed_cloud(seed, abi.ELL_BRENT)
    n = spec.particles.n
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    for chunk in (1, 9, 40):
        h.step(chunk)
        o.step(chunk)
        pg, po = _particles_with_angmom(h, n), o.particles()
        assert_same_particles(pg, po)
        assert np.array_equal(np.nan_to_num(pg.angMom, nan=7.0), np.nan_to_num(po.angMom, nan=7.0)), "angMom differs"
        assert_same_contacts(h.download_contacts(), o.contacts())
    st = h.status()
    assert st.nReal > 10
    assert st.ellSolves > 0
    assert st.nFullRuns == o.n_full_runs()


def test_newton_matches_exact_maximiser(wdem_lib):
    spec = _mixed_cloud(3, abi.ELL_NEWTON)
    n = spec.particles.n
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    h.step(1)
    o.step(1)
    cg, co = h.download_contacts(), o.contacts()
    assert np.array_equal(cg.keys(), co.keys())
    assert np.array_equal(cg.real, co.real)
    assert_same_contacts(cg, co, exact=False, rtol=1e-9)
    assert_same_particles(gpu_particles(h, n), o.particles(), exact=False, rtol=1e-9)
    st = h.status()
    assert st.ellSolves > 0 and 1.0 < st.ellIters / st.ellSolves < 20


@pytest.mark.parametrize("warm", [abi.WARM_COLD, abi.WARM_HISTORY])
def test_newton_warm_starts_agree(wdem_lib, warm):
    """The warm start changes only the iteration count: 30 steps from the same state agree to 1e-9
    with the cold start, and the history start needs fewer iterations per solve."""
    res = {}
    for w in (abi.WARM_COLD, warm):
        spec = _mixed_cloud(4, abi.ELL_NEWTON, warmStart=w)
        h = gpu_handle(spec)
        h.step(30)
        st = h.status()
        res[w] = (gpu_particles(h, spec.particles.n), st.ellIters / max(st.ellSolves, 1))
    pc, ic = res[abi.WARM_COLD]
    pw, iw = res[warm]
    assert np.allclose(pc.pos, pw.pos, rtol=0, atol=1e-9 * np.abs(pc.pos).max())
    if warm == abi.WARM_HISTORY:
        assert iw < ic


@pytest.mark.parametrize("solver", [abi.ELL_BRENT, abi.ELL_NEWTON])
@pytest.mark.parametrize("scale", [0.5 / 3.0, 1.0 / 3.0, 10.0 / 3.0, 100.0 / 3.0, 1000 / 3.0])
def test_normal_displacement_ellipsoid_gpu(wdem_lib, scale, solver):
    """py/tests/test_ellipsoid.py:24-57 on the GPU: overlap 0.01 after one step at every scale."""
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
    h = gpu_handle(scenes.SceneSpec(p, mats, pa))
    h.step(1)
    c = h.download_contacts()
    assert c.n == 1 and c.real[0] == 1
    assert c.uN[0] == pytest.approx(-0.01, abs=1e-5 * 0.01)


def test_free_rotation_bitexact(wdem_lib):
    """Aspherical Leapfrog without contacts: GPU and oracle agree bit for bit (angMom, ori, angVel)."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1e3, young=1e8, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    rng = np.random.default_rng(2)
    k = 50
    centers = np.stack([np.arange(k) * 1.0, np.zeros(k), np.zeros(k)], axis=1)
    semi = rng.uniform(0.1, 0.3, (k, 3))
    pa = scenes.assemble_ellipsoids(centers, semi, scenes.random_quaternions(k, rng), 0, [], mats_py)
    pa.angVel[:] = rng.normal(0, 3.0, (k, 3))
    p = scenes.default_params(mats, dt=1e-4, damping=0.0, verletDist=0.0, trackEnergy=1)
    spec = scenes.SceneSpec(p, mats, pa)
    h = gpu_handle(spec)
    o = bridge.Oracle(p, pa)
    h.step(200)
    o.step(200)
    pg, po = _particles_with_angmom(h, k), o.particles()
    for name in ("pos", "ori", "angVel", "angMom"):
        assert np.array_equal(getattr(pg, name), getattr(po, name)), name
    eg, eo = h.energy(), o.energy()
    assert eg["kinetic"] == pytest.approx(eo["kinetic"], rel=1e-13)
