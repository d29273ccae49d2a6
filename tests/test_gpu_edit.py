"""Particle removal and insertion on the device (wdem_remove_particles, wdem_add_particles) against the
same edits restated on the host for the oracle (download, edit, upload: tests/oracle_handle.py): removed
slots inert and parked, their contacts gone, the forces of the step just run kept; inserted particles in
freed slots and in new slots at the end.  Particles and real contacts must agree bit for bit over the run
that follows (the collider runs in full after each edit on both sides)."""
import numpy as np
import pytest

from woo_gb300 import abi, scenes

from helpers import assert_same_particles, assert_same_real_contacts, gpu_handle, gpu_particles
from oracle_handle import OracleHandle

pytestmark = pytest.mark.gpu


def _pair(spec, cap):
    h = abi.Handle(cap)
    h.keep_geom(False)
    h.set_params(spec.params)
    h.upload_particles(spec.particles)
    h.set_params(spec.params)
    o = OracleHandle(cap)
    o.set_params(spec.params)
    o.upload_particles(spec.particles)
    return h, o


@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_remove_then_add(wdem_lib, law):
    spec = scenes.random_cloud(2000, 17, box=(0.15, 0.15, 0.15), rmin=0.003, rmax=0.005, dense=0.85, law=law)
    n = spec.particles.n
    h, o = _pair(spec, n + 200)
    h.step(60)
    o.step(60)
    # remove 80 particles, among them ones with real contacts
    cg = h.download_contacts()
    touching = np.unique(np.concatenate([cg.idA[cg.real == 1], cg.idB[cg.real == 1]]))
    rng = np.random.default_rng(3)
    ids = np.sort(rng.choice(touching[touching >= 6], 80, replace=False)).astype(np.int32)
    park = np.tile(spec.particles.pos[6 + 1], (len(ids), 1))
    before = h.download_particles(spec.particles.copy())
    h.remove_particles(ids, park)
    o.remove_particles(ids, park)
    for k in (1, 40):
        h.step(k)
        o.step(k)
        assert_same_particles(gpu_particles(h, n), o.download_particles(abi.ParticleArrays(n)))
        assert_same_real_contacts(h.download_contacts(), o.download_contacts())
    assert not np.isin(h.download_contacts().idA, ids).any()
    # insert 50 particles where 50 of the removed ones were (those places are free): 30 into freed slots,
    # 20 appended at the end
    new = before.take(ids[:50])
    new.vel[:] = 0
    new.angVel[:] = 0
    new.force[:] = new.mass[:, None] * np.array([0, 0, -9.81])
    new.torque[:] = 0
    slots = np.concatenate([ids[:30], np.arange(n, n + 20)]).astype(np.int32)
    h.add_particles(new, slots)
    o.add_particles(new, slots)
    m = n + 20
    for k in (1, 60):
        h.step(k)
        o.step(k)
        assert_same_particles(gpu_particles(h, m), o.download_particles(abi.ParticleArrays(m)))
        assert_same_real_contacts(h.download_contacts(), o.download_contacts())
    assert h.status().nReal > 0
    h.close()


def test_edit_argument_errors(wdem_lib):
    spec = scenes.random_cloud(300, 2)
    h = abi.Handle(spec.particles.n + 10)
    h.set_params(spec.params)
    h.upload_particles(spec.particles)
    h.set_params(spec.params)
    h.step(5)
    with pytest.raises(abi.WdemError):
        h.remove_particles([spec.particles.n + 5])
    with pytest.raises(abi.WdemError):
        h.remove_particles([10, 10])
    new = spec.particles.take([20, 21, 22])
    with pytest.raises(abi.WdemError, match="contiguously"):
        h.add_particles(new, [spec.particles.n + 1, spec.particles.n + 2, spec.particles.n + 3])
    h.close()
