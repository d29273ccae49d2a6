"""The oracle's restatement of the scene generator and its OpenMP collider (CPU only).

The CPU arm of the benchmark builds its packings with the oracle's generator so that it never loads the
engine library; both generators must give identical arrays.  The OpenMP build's parallel insertion sort
(InsertionSortCollider.cpp:124-186) must find the same pair set as the serial sort.
"""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes


@pytest.mark.parametrize("n,rmin,rmax,seed", [(500, 0.003, 0.006, 5), (3000, 0.002, 0.006, 2), (800, 0.005, 0.005, 1)])
def test_make_cloud_identical(wdem_lib, n, rmin, rmax, seed):
    lo, hi = np.zeros(3), np.array([0.15, 0.12, 0.3])
    c1, r1 = abi.make_cloud(lo, hi, rmin, rmax, n, seed, max_attempts=400)
    c2, r2 = bridge.make_cloud(lo, hi, rmin, rmax, n, seed, max_attempts=400)
    assert len(r1) > n // 2
    assert np.array_equal(c1, c2) and np.array_equal(r1, r2)


@pytest.mark.parametrize("periodic", [True, False])
@pytest.mark.parametrize("L", [0.021, 0.05, 0.1])
def test_make_cloud_radii_identical(wdem_lib, periodic, L):
    rng = np.random.default_rng(3)
    rin = rng.uniform(0.002, 0.005, 600)
    c1, r1 = abi.make_cloud_radii([0, 0, 0], [L, L, 1.3 * L], rin, 9, periodic=periodic)
    c2, r2 = bridge.make_cloud_radii([0, 0, 0], [L, L, 1.3 * L], rin, 9, periodic=periodic)
    assert np.array_equal(c1, c2) and np.array_equal(r1, r2)
    # no overlap (nearest image when periodic)
    box = np.array([L, L, 1.3 * L])
    d = c1[:, None, :] - c1[None, :, :]
    if periodic:
        d -= box * np.round(d / box)
    dist = np.sqrt((d ** 2).sum(-1))
    rr = r1[:, None] + r1[None, :]
    np.fill_diagonal(dist, np.inf)
    assert (dist >= rr).all()


def test_scene_builder_with_oracle_packer(wdem_lib):
    """The benchmark scene built with either generator is the same scene."""
    a = scenes.hertz1M(n=2000)
    scenes.set_packer(bridge.make_cloud, bridge.make_cloud_radii)
    try:
        b = scenes.hertz1M(n=2000)
    finally:
        scenes.set_packer()
    for name in ("pos", "radius", "mass", "inertia", "material", "shape"):
        assert np.array_equal(getattr(a.particles, name), getattr(b.particles, name), equal_nan=True), name
    assert a.params.dt == b.params.dt


def test_parallel_insertion_sort_pair_set():
    """Serial and OpenMP (chunked odd/even passes, per-thread queues) insertion sorts: same pairs over many
    incremental collider runs of a settling cloud."""
    spec = scenes.random_cloud(6000, 4, box=(0.3, 0.3, 0.3), rmin=0.002, rmax=0.004, dense=0.9)
    spec.params.verletDist = -0.02   # frequent incremental runs
    ser = bridge.Oracle(spec.params, spec.particles, canonical=False, variant="liborc_omp.so")
    par = bridge.Oracle(spec.params, spec.particles, canonical=False, variant="liborc_omp.so")
    par.set_parallel(True)
    ser.step(1)
    par.step(1)
    for _ in range(6):
        ser.step(10)
        par.step(10)
        ks, kp = ser.contacts().keys(), par.contacts().keys()
        # forces are added in thread order in the parallel build, so the trajectories part in the last
        # bits; the pair sets of this short run stay equal
        assert np.array_equal(ks, kp)
    assert ser.n_full_runs() == par.n_full_runs() > 2


def test_parallel_initial_pairs_match_sweep():
    """The OpenMP build's grid search for the initial sort's pairs gives the serial sweep's pair set and
    orientation, walls included, and the same state after further steps."""
    spec = scenes.random_cloud(5000, 8, box=(0.25, 0.25, 0.25), rmin=0.002, rmax=0.004, dense=0.95)
    ser = bridge.Oracle(spec.params, spec.particles, canonical=False, variant="liborc_omp.so")
    par = bridge.Oracle(spec.params, spec.particles, canonical=False, variant="liborc_omp.so")
    par.set_parallel(True)
    ser.step(1)
    par.step(1)
    cs, cp = ser.contacts(), par.contacts()
    assert cs.n > 1000 and np.array_equal(cs.keys(), cp.keys())
    assert np.array_equal(cs.idA, cp.idA) and np.array_equal(cs.idB, cp.idB)
    assert np.array_equal(cs.real, cp.real)


@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_threaded_oracle_is_bitexact(law):
    """The OpenMP build's deterministic loops give the serial oracle's state bit for bit (the long GPU
    parity runs use them)."""
    spec = scenes.random_cloud(3000, 6, box=(0.2, 0.2, 0.2), rmin=0.003, rmax=0.005, dense=0.8, law=law)
    a = bridge.Oracle(spec.params, spec.particles)
    b = bridge.Oracle(spec.params, spec.particles, threads=True)
    for k in (1, 30, 70):
        a.step(k)
        b.step(k)
        pa, pb = a.particles(), b.particles()
        for name in ("pos", "vel", "angVel", "force", "torque", "ori"):
            assert np.array_equal(getattr(pa, name), getattr(pb, name)), name
        ca, cb = a.contacts(), b.contacts()
        assert np.array_equal(ca.keys(), cb.keys()) and np.array_equal(ca.force, cb.force)
    assert int(a.contacts().real.sum()) > 100


def test_threaded_oracle_periodic_bitexact():
    spec = scenes.periodic_cloud(3000, 7, size=(0.09, 0.09, 0.09), rmin=0.002, rmax=0.004, dense=0.8, shear=0.1)
    a = bridge.Oracle(spec.params, spec.particles, cell=spec.cell)
    b = bridge.Oracle(spec.params, spec.particles, cell=spec.cell, threads=True)
    a.step(60)
    b.step(60)
    pa, pb = a.particles(), b.particles()
    for name in ("pos", "vel", "angVel", "force", "torque"):
        assert np.array_equal(getattr(pa, name), getattr(pb, name)), name
    assert np.array_equal(a.stress(), b.stress())
