"""GPU energy tracking (EnergyTracker slots) against the oracle, and the reference's energy tests."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, dem, scenes, utils
from woo_gb300.core import Scene

from helpers import gpu_handle

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_energies_match_oracle(wdem_lib, law):
    """Every slot within 1e-12 relative of the oracle's (sums run in a different order: per-node /
    per-contact terms are the same numbers, the reduction tree differs)."""
    spec = scenes.random_cloud(400, 31, dense=0.85, law=law, trackEnergy=1)
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    h.step(150); o.step(150)
    eg, eo = h.energy(), o.energy()
    assert eo["kinetic"] > 0 and eo["elast"] > 0
    for k in abi.ENERGY_NAMES:
        scale = max(abs(eo[k]), 1e-300)
        assert abs(eg[k] - eo[k]) <= 1e-12 * scale + 1e-300, (k, eg[k], eo[k])


def _energy_scene(flag):
    m = utils.defaultMaterial()
    S = Scene(dtSafety=0.9, trackEnergy=True, engines=dem.DemField.minimalEngines(damping=0.4, dynDtPeriod=0),
              fields=[dem.DemField(gravity=(0, 0, -10), par=[dem.Wall.make(0, axis=2, sense=1, mat=m),
                                                            dem.Sphere.make((0, 0, 0.1), radius=0.8, mat=m)])])
    for n in S.dem.nodes:
        setattr(n.dem, flag, True)
    return S


def test_gravity_skip(wdem_lib):
    """py/tests/test_energy.py:75-82."""
    S = _energy_scene("gravitySkip")
    S.dem.par[-1].vel = (0, 0, -1)
    S.run(400, True)
    assert "grav" not in S.energy
    assert S.energy["nonviscDamp"] != 0.0


def test_damping_skip(wdem_lib):
    """py/tests/test_energy.py:83-90."""
    S = _energy_scene("dampingSkip")
    S.run(400, True)
    assert S.energy["grav"] != 0.0
    assert "nonviscDamp" not in S.energy


def test_energy_balance_elastic(wdem_lib):
    """No damping, frictionless elastic contacts: kinetic + elastic - gravity work stays constant
    (within leapfrog's O(dt) oscillation) over a long bouncing run."""
    spec = scenes.random_cloud(300, 41, dense=0.9, trackEnergy=1, damping=0.0, noFrict=1)
    h = gpu_handle(spec)
    tot = []
    for _ in range(20):
        h.step(100)
        e = h.energy()
        tot.append(e["kinetic"] + e["elast"] + e["grav"])
    tot = np.array(tot)
    assert np.ptp(tot) <= 0.02 * np.abs(tot).max()
