"""Steps queued on the device ahead of the host's collider check (wdem_set_queue_depth): the state after
many steps, with rebuilds in between, is bitwise the same for every queue depth, and the rebuild count
and step counter agree; also against the oracle at the default depth."""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import scenes

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def _run(spec, depth, chunks):
    h = gpu_handle(spec)
    h.set_queue_depth(depth)
    for c in chunks:
        h.step(c)
    return h


@pytest.mark.parametrize("kind", ["frict", "hertz", "ellipsoid", "batch"])
def test_queue_depth_invariance(wdem_lib, kind):
    if kind == "ellipsoid":
        spec = scenes.ellipsoid_cloud(300, 3, dense=0.72, sphere_frac=0.2)
    elif kind == "batch":
        spec = scenes.batch_oedometric(4, 3, nmin=150, nmax=400, dense=0.85)
    else:
        spec = scenes.random_cloud(600, 2, dense=0.8, law=kind)
    n = spec.particles.n
    chunks = (1, 7, 100, 292)
    ref = _run(spec, 1, chunks)
    pr, cr, sr = gpu_particles(ref, n), ref.download_contacts(), ref.status()
    assert sr.nFullRuns >= 3, "the scene should rebuild its pair set a few times"
    for depth in (2, 3, 32, 200):
        h = _run(spec, depth, chunks)
        assert_same_particles(gpu_particles(h, n), pr, ori_tol=0)
        assert_same_contacts(h.download_contacts(), cr)
        st = h.status()
        assert st.step == sr.step == sum(chunks)
        assert st.nFullRuns == sr.nFullRuns


def test_queued_against_oracle(wdem_lib):
    spec = scenes.random_cloud(500, 9, dense=0.85, law="hertz")
    n = spec.particles.n
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    for c in (1, 60, 240):
        h.step(c)
        o.step(c)
        assert_same_particles(gpu_particles(h, n), o.particles())
        assert_same_contacts(h.download_contacts(), o.contacts())
    assert h.status().nFullRuns == o.n_full_runs()


def test_queue_depth_argument_checked(wdem_lib):
    spec = scenes.random_cloud(50, 1)
    h = gpu_handle(spec)
    with pytest.raises(Exception):
        h.set_queue_depth(-1)
    h.set_queue_depth(0)
    h.step(5)
    assert h.status().step == 5
