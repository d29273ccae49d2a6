"""Woo-style scripts through the Python surface on the GPU, checked against the oracle."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, dem, utils
from woo_gb300.core import Scene

pytestmark = pytest.mark.gpu


def test_sphere_on_wall_script(wdem_lib):
    """py/tests/test_energy.py's scene (wall + sphere, gravity -10, damping .4, dtSafety .9) through
    Scene/DemField/minimalEngines: same trajectory as the oracle, bit for bit."""
    m = utils.defaultMaterial()
    S = Scene(dtSafety=0.9, engines=dem.DemField.minimalEngines(damping=0.4, dynDtPeriod=0),
              fields=[dem.DemField(gravity=(0, 0, -10), par=[dem.Wall.make(0, axis=2, sense=1, mat=m),
                                                            dem.Sphere.make((0, 0, 0.1), radius=0.8, mat=m)])])
    S.dem.par[-1].vel = (0, 0, -1)
    S._prepare_dt()
    g = S._engine()
    params = g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    o = bridge.Oracle(params, pa)
    S.run(400)
    o.step(400)
    po = o.particles()
    assert np.array_equal(S.dem.par[1].pos, po.pos[1])
    assert np.array_equal(S.dem.par[1].vel, po.vel[1])
    assert S.step == 400
    assert len(S.dem.con) == o.contacts().n


def test_update_phys_script(wdem_lib):
    """py/tests/test_demfield.py:24-51 verbatim in spirit, via the Python surface."""
    for up in ("never", "always", "once"):
        E0, E1 = 1e3, 1e6
        m = dem.FrictMat(young=E0)
        S = Scene(fields=[dem.DemField(par=[dem.Sphere.make((0, 0, 0), 0.6, mat=m), dem.Sphere.make((0, 0, 1), 0.6, mat=m)])],
                  engines=dem.DemField.minimalEngines(dynDtPeriod=0), dtSafety=1e-8, dt=1e-8)
        S.one()
        c = S.dem.con[0]
        kn0 = c.phys.kn
        S.lab.contactLoop.updatePhys = up
        m.young = E1
        S.one()
        kn1 = S.dem.con[0].phys.kn
        if up in ("always", "once"):
            assert kn1 == pytest.approx(kn0 * (E1 / E0))
        else:
            assert kn1 == pytest.approx(kn0)
        m.young = E0
        S.one()
        if up == "always":
            assert S.lab.contactLoop.updatePhys == "always"
            assert S.dem.con[0].phys.kn == pytest.approx(kn0)
        else:
            assert S.lab.contactLoop.updatePhys == "never"
            assert S.dem.con[0].phys.kn == kn1


def test_edit_state_between_runs(wdem_lib):
    """Writing a particle's velocity between runs reaches the GPU without losing contact history."""
    m = dem.FrictMat(density=2500, young=1e7)
    par = [dem.Wall.make(0, axis=2, sense=1, mat=m), dem.Sphere.make((0, 0, 0.009999), 0.01, mat=m)]
    S = Scene(fields=[dem.DemField(gravity=(0, 0, -9.81), par=par)], engines=dem.DemField.minimalEngines(dynDtPeriod=0))
    S.run(1)
    assert S.dem.con.countReal() == 1
    c = S.dem.con[(0, 1)]
    assert c.real and c.geom.uN < 0 and c.forceSign(0) == 1 and c.forceSign(1) == -1
    S.dem.par[1].vel = (0.1, 0, 0)
    S.run(1)
    assert S.dem.par[1].vel[0] > 0.05
    assert S.dem.con.countReal() == 1
