"""GPU engine vs the oracle at the benchmark configurations (or cuts of them where the oracle would take
too long), through the C ABI.

- the 10,000-sphere FrictMat scene in full: 2000 steps, bit-exact;
- a 100,000-sphere cut of the 1M Hertz-DMT workload (same density, box scaled): falling for 300 steps,
  and settled on the GPU first with the settled state (particles and contacts with history) uploaded to
  both sides, 100 steps; bit-exact;
- a 10,000-sphere cut of the periodic simple-shear workload (lognormal radii, densified to solid fraction
  0.62), stress tensor compared every 1000 steps over 3000 steps (ContactLoop.cpp:218-254), state
  bit-exact at the end;
- a 1,500-ellipsoid cut of the ellipsoid workload with the reference's Brent solver, 200 steps, bit-exact
  (orientations and angular momentum to 1e-12: sin/cos differ in the last bit between CUDA and the C
  library);
- four oedometric scenes of the batched workload run as one GPU batch, each compared with the oracle
  running that scene alone with its moving top wall: particle state bit-exact, real contacts and their
  forces equal.

Bit-exact bar: both sides run the same IEEE operations in the same order.  The larger runs use the
oracle's OpenMP build in its deterministic mode (the serial oracle's results bit for bit, checked in
tests/test_oracle_pack.py).
"""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes

from helpers import assert_same_contacts, assert_same_particles, assert_same_real_contacts, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def _compare(h, o, n, cell=False):
    assert_same_particles(gpu_particles(h, n), o.particles())
    cg, co = h.download_contacts(), o.contacts()
    assert_same_contacts(cg, co)
    if cell:
        assert np.array_equal(cg.cellDist, co.cellDist), "cellDist differs"
    return cg


def test_spheres10k_full_run(wdem_lib):
    spec = scenes.spheres10k()
    n = spec.particles.n
    h = gpu_handle(spec, keep_geom=False)
    o = bridge.Oracle(spec.params, spec.particles, threads=True)
    for chunk in (1, 499, 500, 1000):
        h.step(chunk)
        o.step(chunk)
    cg = _compare(h, o, n)
    assert h.status().nFullRuns == o.n_full_runs()
    assert int(cg.real.sum()) > 0, "spheres near the floor reach it within the run"


def test_hertz100k_falling(wdem_lib):
    spec = scenes.hertz1M(n=100_000)
    n = spec.particles.n
    h = gpu_handle(spec, keep_geom=False)
    o = bridge.Oracle(spec.params, spec.particles, threads=True)
    for chunk in (5, 295):
        h.step(chunk)
        o.step(chunk)
        _compare(h, o, n)
    assert h.status().nFullRuns == o.n_full_runs()


def test_hertz100k_settled(wdem_lib):
    spec = scenes.hertz1M(n=100_000, height=0.95)
    n = spec.particles.n
    hs = gpu_handle(spec, keep_geom=False)
    scenes.settle(hs, spec, tail_steps=1000)
    # the downloaded dynamic state over a copy of the scene's static arrays (radius, mass, material, ...)
    pa = hs.download_particles(spec.particles.copy())
    ca = hs.download_contacts()
    step = hs.status().step
    hs.close()
    assert int(ca.real.sum()) > 50_000, "settled packing: about one real contact per sphere or more"
    p = scenes.copy_params(spec.params)
    p.step = step
    h = abi.Handle(n)
    h.set_params(p)
    h.upload_particles(pa)
    h.set_params(p)
    h.upload_contacts(ca)
    o = bridge.Oracle(p, pa, contacts=ca, threads=True)
    for chunk in (1, 99):
        h.step(chunk)
        o.step(chunk)
        assert_same_particles(gpu_particles(h, n), o.particles())
        cg = h.download_contacts()
        assert_same_real_contacts(cg, o.contacts())
    assert int(cg.real.sum()) > 50_000


def test_peri10k_stress_every_1000(wdem_lib):
    spec = scenes.densify_periodic(scenes.peri_shear(n=10_000), phi_target=0.62)
    n = spec.particles.n
    h = gpu_handle(spec, keep_geom=False)
    o = bridge.Oracle(spec.params, spec.particles, cell=spec.cell, threads=True)
    for k in range(3):
        h.step(1000)
        o.step(1000)
        sg, so = h.stress(), o.stress()
        assert np.abs(so).max() > 0
        # the sum runs in a different order on the two sides: relative 1e-12 of the largest component
        assert np.allclose(sg, so, rtol=0, atol=1e-12 * np.abs(so).max()), (k, sg, so)
    cg = _compare(h, o, n, cell=True)
    assert int(cg.real.sum()) > 10_000


def test_ellipsoids_brent_cut(wdem_lib):
    spec = scenes.ellipsoid_cloud(1500, 7, box=(0.09, 0.09, 0.18), amin=0.003, amax=0.006, dense=0.8,
                                  vel_scale=0.5, angvel_scale=5.0, young=1e7, tanPhi=0.4, damping=0.2,
                                  ellSolver=abi.ELL_BRENT)
    n = spec.particles.n
    h = gpu_handle(spec, keep_geom=False)
    o = bridge.Oracle(spec.params, spec.particles)
    for chunk in (1, 49, 150):
        h.step(chunk)
        o.step(chunk)
    pg, po = gpu_particles(h, n), o.particles()
    for name in ("pos", "vel", "force", "torque"):
        assert np.array_equal(getattr(pg, name), getattr(po, name)), name
    assert np.allclose(pg.ori, po.ori, rtol=0, atol=1e-12)
    assert np.allclose(pg.angVel, po.angVel, rtol=1e-12, atol=1e-12 * np.abs(po.angVel).max())
    cg, co = h.download_contacts(), o.contacts()
    assert np.array_equal(cg.keys(), co.keys()) and np.array_equal(cg.real, co.real)
    assert int(cg.real.sum()) > 20


def test_batch_scenes_against_oracle(wdem_lib):
    spec = scenes.batch_oedometric(4, 9, nmin=400, nmax=1500, dense=0.9)
    n = spec.particles.n
    hb = gpu_handle(spec, keep_geom=False)
    steps = 400
    hb.step(steps)
    pb = gpu_particles(hb, n)
    cb = hb.download_contacts()
    for k in range(4):
        a, b = spec.info["ranges"][k]
        single = scenes.single_from_batch(spec, k)
        o = bridge.Oracle(single.params, single.particles)
        o.step(steps)
        po = o.particles()
        for name in ("pos", "vel", "angVel", "force", "torque"):
            assert np.array_equal(getattr(pb, name)[a:b], getattr(po, name)), (k, name)
        assert np.allclose(pb.ori[a:b], po.ori, rtol=0, atol=1e-12)
        # the moving top wall (index 5 of each scene) went down at 0.05 m/s
        assert po.pos[5, 2] < single.particles.pos[5, 2]
        co = o.contacts()
        sel = (cb.idA >= a) & (cb.idA < b) & (cb.real == 1)
        kb = np.minimum(cb.idA[sel] - a, cb.idB[sel] - a).astype(np.int64) * 1_000_000 + np.maximum(cb.idA[sel] - a, cb.idB[sel] - a)
        ro = co.real == 1
        ko = co.keys()[ro]
        kb2 = (kb // 1_000_000 << 32) | (kb % 1_000_000)
        ob, oo = np.argsort(kb2), np.argsort(ko)
        assert np.array_equal(kb2[ob], ko[oo]), k
        assert int(ro.sum()) >= 10, k
        assert np.array_equal(cb.force[sel][ob], co.force[ro][oo]), k
