"""Queued steps replayed from CUDA graphs (wdem_set_step_graphs): the state after many steps, with
rebuilds, parameter changes and uploads in between, is bitwise the same as with every kernel launched
from the host, and the graph path matches the oracle; graphs are captured again whenever a launch
argument changed, and the launch count covers the kernels of every replay."""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def _spec(kind):
    if kind == "ellipsoid":
        return scenes.ellipsoid_cloud(300, 3, dense=0.72, sphere_frac=0.2, ellSolver=abi.ELL_NEWTON,
                                      warmStart=abi.WARM_HISTORY)
    if kind == "ellipsoid_mlp":
        return scenes.ellipsoid_cloud(300, 4, dense=0.72, ellSolver=abi.ELL_NEWTON, warmStart=abi.WARM_HISTORY_MLP)
    if kind == "batch":
        return scenes.batch_oedometric(4, 3, nmin=150, nmax=400, dense=0.85)
    return scenes.random_cloud(600, 2, dense=0.8, law=kind)


def _run(spec, mode, chunks, kind=""):
    h = gpu_handle(spec)
    if kind == "ellipsoid_mlp":
        h.warm_init(7)
    h.set_step_graphs(mode)
    l0 = h.launch_count()
    for c in chunks:
        h.step(c)
    return h, h.launch_count() - l0


@pytest.mark.parametrize("kind", ["frict", "hertz", "ellipsoid", "ellipsoid_mlp", "batch"])
def test_graphs_bitwise_as_launches(wdem_lib, kind):
    spec = _spec(kind)
    n = spec.particles.n
    chunks = (1, 7, 100, 292)
    ref, lref = _run(spec, abi.GRAPHS_OFF, chunks, kind)
    pr, cr, sr = gpu_particles(ref, n), ref.download_contacts(), ref.status()
    assert ref.graph_stats() == (0, 0)
    h, lg = _run(spec, abi.GRAPHS_ON, chunks, kind)
    assert_same_particles(gpu_particles(h, n), pr, ori_tol=0)
    assert_same_contacts(h.download_contacts(), cr)
    st = h.status()
    assert st.step == sr.step == sum(chunks)
    assert st.nFullRuns == sr.nFullRuns
    captures, replays = h.graph_stats()
    assert captures > 0 and replays >= captures
    # the same kernels ran: a replay counts the kernels its graph holds
    assert lg == lref


def test_graphs_against_oracle(wdem_lib):
    spec = scenes.random_cloud(500, 9, dense=0.85, law="hertz")
    n = spec.particles.n
    h = gpu_handle(spec)
    h.set_step_graphs(abi.GRAPHS_ON)
    o = bridge.Oracle(spec.params, spec.particles)
    for c in (1, 60, 240):
        h.step(c)
        o.step(c)
        assert_same_particles(gpu_particles(h, n), o.particles())
        assert_same_contacts(h.download_contacts(), o.contacts())
    assert h.status().nFullRuns == o.n_full_runs()
    assert h.graph_stats()[1] > 0


def test_graphs_recaptured_on_changes(wdem_lib):
    """New parameters (damping, dt) and a re-uploaded state between calls: the replays use the new
    arguments, as the kernel-by-kernel path does."""
    spec = scenes.random_cloud(400, 5, dense=0.8, law="frict")
    n = spec.particles.n
    runs = []
    for mode in (abi.GRAPHS_OFF, abi.GRAPHS_ON):
        h = gpu_handle(spec)
        h.set_step_graphs(mode)
        h.step(80)
        p = scenes.copy_params(spec.params)
        p.damping = 0.05
        p.dt = spec.params.dt * 0.7
        p.step = h.status().step
        h.set_params(p)
        h.step(120)
        state = h.download_particles(spec.particles.copy())   # static fields from the scene, state from the GPU
        contacts = h.download_contacts()
        h.upload_particles(state)
        h.upload_contacts(contacts)
        h.step(150)
        runs.append((gpu_particles(h, n), h.download_contacts(), h.status().step, h.graph_stats()))
    (p0, c0, s0, g0), (p1, c1, s1, g1) = runs
    assert_same_particles(p1, p0, ori_tol=0)
    assert_same_contacts(c1, c0)
    assert s0 == s1 == 350
    assert g0 == (0, 0) and g1[0] >= 2


def test_graph_mode_argument_checked(wdem_lib):
    spec = scenes.random_cloud(50, 1)
    h = gpu_handle(spec)
    for bad in (-1, 3):
        with pytest.raises(Exception):
            h.set_step_graphs(bad)
    h.set_step_graphs(abi.GRAPHS_AUTO)
    h.step(5)
    assert h.status().step == 5
