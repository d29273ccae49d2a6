"""Inlets on the GPU engine against the same scripts run on the oracle: the spheres an inlet places (the
placement reads the positions of the particles already in the scene), with an outlet freeing ids for
it, and the scene that follows."""
import numpy as np
import pytest

from woo_gb300 import dem

from oracle_handle import run_on_oracle
from test_gpu_outlet import _compare
from test_inlet import bin_scene, inlet

pytestmark = [pytest.mark.gpu, pytest.mark.host_engines]


def _pair(**kw):
    out = []
    for _ in range(2):
        S, m = bin_scene(n_pre=20, trackEnergy=True)
        ii = inlet(m, massRate=1.0, maxNum=40, seed=11,
                   shooter=dem.AlignedMinMaxShooter(dir=(0, 0, -1), vRange=(0.1, 0.5)), **kw)
        S.engines = S.engines + [ii]
        out.append((S, ii))
    return out


def test_inlet_matches_oracle(wdem_lib, monkeypatch):
    (Sg, ig), (So, io) = _pair()
    Sg.run(1501)
    run_on_oracle(monkeypatch, So, 1501)
    assert ig.num == io.num == 40 and ig.mass == io.mass
    assert len(Sg.dem.par) == len(So.dem.par)
    assert Sg._gpu._cap >= len(Sg.dem.par)
    _compare(Sg, So, len(Sg.dem.par))
    assert Sg.energy["kinInlet"] == So.energy["kinInlet"]


def test_inlet_into_freed_ids_matches_oracle(wdem_lib, monkeypatch):
    runs = []
    for run in (lambda S, n: S.run(n), lambda S, n: run_on_oracle(monkeypatch, S, n)):
        S, m = bin_scene(n_pre=10, gravity=(0, 0, -9.81))
        S.dem.par[7].pos = (0.0, 0.0, -0.5)
        S.dem.par[9].pos = (0.01, 0.0, -0.5)
        out = dem.BoxOutlet(box=((-1, -1, -0.1), (1, 1, 1)), stepPeriod=50)
        ii = inlet(m, massRate=0.5, maxNum=3, seed=4, stepPeriod=100)
        S.engines = S.engines + [out, ii]
        run(S, 801)
        runs.append((S, out, ii))
    (Sg, og, ig), (So, oo, io) = runs
    assert og.num == oo.num == 2 and ig.num == io.num == 3
    _compare(Sg, So, len(So.dem.par))
