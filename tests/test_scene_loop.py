"""Scene loop semantics of py/tests/test_core.py:291-376 that apply to a synchronous GPU engine:
stopAtStep / run(steps=...), stopAtTime / run(time=...), dead engines, steps=0; on the CPU."""
import math

import pytest

from woo_gb300 import dem
from woo_gb300.core import Scene

from oracle_handle import run_on_oracle
from test_outlet import funnel


def test_stop_at_step():
    """test_core.py:360-366."""
    S = Scene(dt=1.)
    S.stopAtStep = 100                                    # absolute value
    S.run(wait=True)
    assert S.step == 100
    S.run(steps=100, wait=True)                           # relative value
    assert S.step == 200
    with pytest.raises(RuntimeError, match="nothing to run"):
        S.run(wait=True)                                  # stopAtStep already reached


def test_stop_at_time():
    """test_core.py:367-374."""
    S = Scene(dt=1e-3)
    S.stopAtTime = 1.0001                                 # absolute value
    S.run(wait=True)
    assert S.time == pytest.approx(1.001, abs=1e-3)
    S.run(time=.5, wait=True)                             # relative value
    assert S.time == pytest.approx(1.501, abs=1e-3)


def test_stop_at_time_with_the_gpu_engine(monkeypatch):
    """The run ends after the first step that brings the time to stopAtTime, also when it is split into
    chunks around host engines."""
    out = dem.BoxOutlet(box=((-1, -1, -1), (1, 1, 10)), stepPeriod=37)
    S = funnel(engines=[out])
    S._prepare_dt()
    goal = 250.5 * S.dt
    with monkeypatch.context() as m:
        from woo_gb300 import abi
        from oracle_handle import OracleHandle
        m.setattr(abi, "Handle", OracleHandle)
        S.run(time=goal)
    assert S.time >= goal and S.time - S.dt < goal
    assert S.step == 251
    assert out.nDone == 251 // 37 + 1


def test_dead_engine_not_run(monkeypatch):
    """test_core.py:335-339."""
    out = dem.BoxOutlet(box=((-1, -1, -1), (1, 1, 1)), stepPeriod=1, dead=True)
    S = funnel(engines=[out])
    run_on_oracle(monkeypatch, S, 3)
    assert out.nDone == 0


def test_zero_steps_and_hooks():
    S = Scene(dt=1.)
    S.run(0)
    assert S.step == 0
    S.stopAtHook = "S.lab.a+=1"
    with pytest.raises(RuntimeError, match="stopAtHook"):
        S.run(5)


def test_save_tmp_load_tmp(monkeypatch):
    """Scene.saveTmp / loadTmp (py/tests/test_io.py:105-111): a copy from memory continues like the original."""
    S = funnel(floor=True)
    run_on_oracle(monkeypatch, S, 200)
    S.saveTmp("a")
    T = Scene.loadTmp("a")
    run_on_oracle(monkeypatch, S, 300)
    run_on_oracle(monkeypatch, T, 300)
    assert T.step == S.step == 500 and T.time == S.time
    for p in S.dem.par:
        assert (p.pos == T.dem.par[p.id].pos).all() and (p.vel == T.dem.par[p.id].vel).all()
    with pytest.raises(ValueError):
        Scene.loadTmp("missing")


def test_synchronous_loop_controls():
    S = Scene(dt=1.)
    with S.paused():
        assert not S.running
    S.run(3)
    S.stop()
    S.wait()
    assert S.step == 3 and not S.running
