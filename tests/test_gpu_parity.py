"""GPU engine vs the CPU oracle on identical seeded scenes.

Bar: bit-exact particle state (pos, vel, angVel, force, torque) and contact history (pair set,
orientation, trsf, contact point, local force, stiffnesses) over many steps, because both sides run
the same IEEE operations in the same order (no FMA contraction on either side).  Sphere
orientations go through sin/cos, where CUDA and the C library may differ by an ulp: 1e-12 there.
"""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("law", ["frict", "hertz"])
@pytest.mark.parametrize("seed", [1, 2])
def test_multistep_bitexact(wdem_lib, law, seed):
    spec = scenes.random_cloud(400, seed, dense=0.85, law=law)
    n = spec.particles.n
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    for chunk in (1, 4, 45, 150):
        h.step(chunk)
        o.step(chunk)
        assert_same_particles(gpu_particles(h, n), o.particles())
        assert_same_contacts(h.download_contacts(), o.contacts())
    st = h.status()
    assert st.nFullRuns == o.n_full_runs()
    assert st.nReal > 0


def test_no_gravity_no_damping(wdem_lib):
    spec = scenes.random_cloud(200, 5, dense=0.8, gravity=(0, 0, 0), damping=0.0)
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    h.step(100); o.step(100)
    assert_same_particles(gpu_particles(h, spec.particles.n), o.particles())
    assert_same_contacts(h.download_contacts(), o.contacts())
