"""Engine-state checkpoints (woo_gb300.checkpoint): the archive round trip, and a run saved halfway and
resumed (a fresh engine, full collider run on the first step, as after the reference's Scene.load)
that continues bit for bit like the uninterrupted run; exercised on the oracle, which takes the same
particle and contact arrays as the GPU engine."""
import ctypes

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, checkpoint, scenes

DYN = ("pos", "vel", "angVel", "ori", "force", "torque", "angMom")


def _state(o, static):
    pa = static.copy()
    q = o.particles()
    for k in DYN:
        setattr(pa, k, getattr(q, k).copy())
    return pa


def test_archive_round_trip(tmp_path):
    spec = scenes.random_cloud(120, 3, dense=0.85, law="hertz")
    o = bridge.Oracle(spec.params, spec.particles)
    o.step(20)
    pa, ca = _state(o, spec.particles), o.contacts()
    cell = dict(hSize=np.diag([1.0, 2, 3]), trsf=np.eye(3), gradV=np.zeros((3, 3)), nextGradV=np.ones((3, 3)))
    path = tmp_path / "s.npz"
    checkpoint.save_state(path, pa, ca, 20, spec.params.dt, cell)
    s = checkpoint.load_state(path)
    assert s["step"] == 20 and s["dt"] == spec.params.dt
    for k, v in pa.__dict__.items():
        if isinstance(v, np.ndarray):
            assert np.array_equal(getattr(s["particles"], k), v, equal_nan=True), k
    for k, v in ca.__dict__.items():
        if isinstance(v, np.ndarray):
            assert np.array_equal(getattr(s["contacts"], k), v, equal_nan=True), k
    assert np.array_equal(s["cell"]["nextGradV"], np.ones((3, 3)))


def test_wrong_format_is_rejected(tmp_path):
    path = tmp_path / "x.npz"
    np.savez(path, format=np.array("something else"), version=np.array(1))
    with pytest.raises(ValueError):
        checkpoint.load_state(path)


@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_resume_continues_exactly(tmp_path, law):
    spec = scenes.random_cloud(300, 8, dense=0.85, law=law)
    whole = bridge.Oracle(spec.params, spec.particles)
    whole.step(150)
    first = bridge.Oracle(spec.params, spec.particles)
    first.step(70)
    path = tmp_path / "half.npz"
    checkpoint.save_state(path, _state(first, spec.particles), first.contacts(), 70, spec.params.dt)
    s = checkpoint.load_state(path)
    p = abi.Params()
    ctypes.memmove(ctypes.byref(p), ctypes.byref(spec.params), ctypes.sizeof(p))
    p.step, p.dt = s["step"], s["dt"]
    second = bridge.Oracle(p, s["particles"], contacts=s["contacts"])
    second.step(80)
    a, b = whole.particles(), second.particles()
    for k in ("pos", "vel", "angVel", "force", "torque"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    ca, cb = whole.contacts(), second.contacts()
    ra, rb = ca.real == 1, cb.real == 1
    assert np.array_equal(np.sort(ca.keys()[ra]), np.sort(cb.keys()[rb]))
    oa, ob = np.argsort(ca.keys()[ra]), np.argsort(cb.keys()[rb])
    assert np.array_equal(ca.force[ra][oa], cb.force[rb][ob])



def test_resume_sheared_periodic(tmp_path):
    """A sheared periodic cell under simple shear, saved halfway and resumed, continues bit for bit.  The
    archive holds hSize, trsf, gradV and nextGradV but not Cell.pprevHsize: every step starts with
    Cell::integrateAndUpdate (src/core/Scene.cpp:411), which sets pprevHsize = (previous + new hSize) / 2
    before the contact loop reads it (Cell::intrShiftVel, src/core/Cell.cpp:31), so the value a resumed
    handle starts with (hSize, as after the reference's Scene.load) is never used."""
    spec = scenes.periodic_cloud(300, 4, dense=0.85)
    whole = bridge.Oracle(spec.params, spec.particles, cell=spec.cell)
    whole.step(150)
    first = bridge.Oracle(spec.params, spec.particles, cell=spec.cell)
    first.step(70)
    cell = first.cell()
    assert not np.array_equal(cell["pprevHsize"], cell["hSize"])
    c = first.contacts()
    assert np.any(c.cellDist[c.real == 1] != 0)
    path = tmp_path / "half.npz"
    checkpoint.save_state(path, _state(first, spec.particles), c, 70, spec.params.dt, cell)
    s = checkpoint.load_state(path)
    p = scenes.copy_params(spec.params)
    p.step, p.dt = s["step"], s["dt"]
    second = bridge.Oracle(p, s["particles"], contacts=s["contacts"], cell=s["cell"])
    second.step(80)
    a, b = whole.particles(), second.particles()
    for k in ("pos", "vel", "angVel", "force", "torque"):
        assert np.array_equal(getattr(a, k), getattr(b, k)), k
    assert np.array_equal(whole.cell()["hSize"], second.cell()["hSize"])
