"""Outlets on the GPU engine against the same scripts run on the oracle: the particles an outlet removes
or marks, its mass bookkeeping, and the state of the scene that continues after the removals."""
import numpy as np
import pytest

from woo_gb300 import dem

from oracle_handle import run_on_oracle
from test_outlet import funnel

pytestmark = [pytest.mark.gpu, pytest.mark.host_engines]


def _compare(Sg, So, n0):
    live_g = [i for i in range(n0) if Sg.dem.par.exists(i)]
    live_o = [i for i in range(n0) if So.dem.par.exists(i)]
    assert live_g == live_o
    for i in live_g:
        for name in ("pos", "vel", "angVel"):
            a, b = getattr(Sg.dem.par[i], name), getattr(So.dem.par[i], name)
            assert np.allclose(a, b, rtol=1e-12, atol=1e-15), (i, name, a, b)
    cg, co = Sg.dem._contacts(), So.dem._contacts()
    rg, ro = cg.real.astype(bool), co.real.astype(bool)
    assert np.array_equal(cg.keys()[rg], co.keys()[ro])
    for name in ("force", "trsf", "contPt", "kn", "kt"):
        a, b = getattr(cg, name)[rg], getattr(co, name)[ro]
        scale = np.abs(b).max() if b.size else 1.0
        assert np.allclose(a, b, rtol=1e-12, atol=1e-12 * scale), name


def test_box_outlet_matches_oracle(wdem_lib, monkeypatch):
    outs = [dem.BoxOutlet(box=((-1, -1, -0.05), (1, 1, 10)), stepPeriod=50, save=True) for _ in range(2)]
    Sg, So = funnel(engines=[outs[0]]), funnel(engines=[outs[1]])
    n0 = len(Sg.dem.par)
    Sg.run(1201)
    run_on_oracle(monkeypatch, So, 1201)
    og, oo = outs
    assert og.num == oo.num > 5
    assert og.mass == oo.mass
    assert og.diamMassTime(zipped=True) == oo.diamMassTime(zipped=True)
    _compare(Sg, So, n0)


def test_outlet_then_settled_column_matches_oracle(wdem_lib, monkeypatch):
    """Removal while ~70 contacts are real, then 600 more steps of the column on the floor."""
    outs = [dem.BoxOutlet(box=((-5, -5, -1), (5, 5, 10)), stepPeriod=300, initRun=False) for _ in range(2)]
    Sg = funnel(floor=True, layers=6, extra=[(3.0, 0, -0.70)], engines=[outs[0]])
    So = funnel(floor=True, layers=6, extra=[(3.0, 0, -0.70)], engines=[outs[1]])
    n0 = len(Sg.dem.par)
    Sg.run(2701)
    run_on_oracle(monkeypatch, So, 2701)
    assert outs[0].num == outs[1].num == 1 and not Sg.dem.par.exists(n0 - 1)
    assert Sg.dem.con.countReal() > 50
    _compare(Sg, So, n0)


def test_marking_and_energy_match_oracle(wdem_lib, monkeypatch):
    outs = [dem.BoxOutlet(box=((-1, -1, -0.05), (1, 1, 10)), stepPeriod=40, markMask=16) for _ in range(2)]
    dels = [dem.BoxOutlet(box=((-1, -1, -0.12), (1, 1, 10)), stepPeriod=70) for _ in range(2)]
    Sg, So = funnel(engines=[outs[0], dels[0]]), funnel(engines=[outs[1], dels[1]])
    Sg.trackEnergy = So.trackEnergy = True
    n0 = len(Sg.dem.par)
    Sg.run(1401)
    run_on_oracle(monkeypatch, So, 1401)
    assert outs[0].num == outs[1].num > 3 and dels[0].num == dels[1].num > 3
    assert [p.mask for p in Sg.dem.par] == [p.mask for p in So.dem.par]
    eg, eo = Sg.energy, So.energy
    assert eg["kinOutlet"] == pytest.approx(eo["kinOutlet"], rel=1e-12)
    _compare(Sg, So, n0)
