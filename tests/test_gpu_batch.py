"""Batched independent scenes (one particle set, scene index per particle, per-scene dt through
wdem_params.materialDt): every scene of the batch evolves exactly as the same scene run alone."""
import numpy as np
import pytest

from woo_gb300 import abi, scenes

from helpers import gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def test_batch_equals_scene_by_scene(wdem_lib):
    spec = scenes.batch_oedometric(5, 3, nmin=150, nmax=600, dense=0.85)
    n = spec.particles.n
    hb = gpu_handle(spec)
    steps = 300
    hb.step(steps)
    pb = gpu_particles(hb, n)
    cb = hb.download_contacts()
    assert hb.status().nReal > 20
    for k in range(5):
        a, b = spec.info["ranges"][k]
        single = scenes.single_from_batch(spec, k)
        hs = gpu_handle(single)
        hs.step(steps)
        ps = gpu_particles(hs, b - a)
        for name in ("pos", "vel", "angVel", "force", "torque"):
            assert np.array_equal(getattr(pb, name)[a:b], getattr(ps, name)), (k, name)
        assert np.allclose(pb.ori[a:b], ps.ori, rtol=0, atol=1e-12)
        # real contacts and their forces agree; potential pairs may differ, because the batch rebuilds its
        # collider whenever any of its scenes triggers it (a potential pair carries no physics)
        cs = hs.download_contacts()
        sel = (cb.idA >= a) & (cb.idA < b) & (cb.real == 1)
        kb = (cb.idA[sel] - a).astype(np.int64) * 1_000_000 + (cb.idB[sel] - a)
        rs = cs.real == 1
        ks = cs.idA[rs].astype(np.int64) * 1_000_000 + cs.idB[rs]
        ob, os_ = np.argsort(kb), np.argsort(ks)
        assert np.array_equal(kb[ob], ks[os_]), k
        assert np.array_equal(cb.force[sel][ob], cs.force[rs][os_]), k
    # no contact joins two scenes
    scene = spec.particles.scene
    assert np.all(scene[cb.idA] == scene[cb.idB])


def test_batch_top_wall_moves(wdem_lib):
    spec = scenes.batch_oedometric(3, 5, nmin=200, nmax=400)
    h = gpu_handle(spec)
    h.step(200)
    p = gpu_particles(h, spec.particles.n)
    for k, (a, b) in enumerate(spec.info["ranges"]):
        top = a + 5
        z0 = spec.particles.pos[top, 2]
        expected = z0 - 0.05 * 200 * spec.info["dt"][k]
        assert p.pos[top, 2] == pytest.approx(expected, rel=1e-12)
