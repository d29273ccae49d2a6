"""DynDt in the oracle (src/dem/DynDt.cpp:16-113): the critical step of two touching FrictMat spheres
against its closed form, the PeriodicEngine schedule (stepPeriod with stepModulo) and the growth cap
dt (1 + maxRelInc)^n."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes


def _pair(dt, period, maxRelInc=1e-4, dtSafety=0.9):
    mats_py = [dict(kind=abi.MAT_FRICT, density=2000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    r = 0.01
    pa = scenes.assemble(np.array([[0.0, 0, 0], [2 * r - 1e-5, 0, 0]]), np.array([r, r]), 0, [], mats_py)
    p = scenes.default_params(mats, dt=dt, gravity=(0, 0, 0), damping=0.0)
    p.dynDtPeriod = period
    p.dynDtMaxRelInc = maxRelInc
    p.dtSafety = dtSafety
    m = float(pa.mass[0])
    kn = 1e7 * math.pi * r * r / (2 * r)  # 1/(1/(E A/r) + 1/(E A/r)), A = pi r^2
    return bridge.Oracle(p, pa), mats, m, kn


def test_two_spheres_critical_step():
    o, mats, m, kn = _pair(dt=1.0, period=1)
    o.step(1)
    crit = math.sqrt(2 * m / kn)  # min over m/kn, m/kt, I/(r^2 kt) = 2 m/kn times 2, then sqrt
    assert o.dyndt_crit() == pytest.approx(crit, rel=1e-12)
    # first run: no growth allowed yet (n = 0), so dt drops to dtSafety x the critical step
    assert o.dt() == pytest.approx(0.9 * crit, rel=1e-12)


def test_growth_cap_and_schedule():
    o, mats, m, kn = _pair(dt=1e-7, period=5, maxRelInc=1e-3)
    dts = []
    for k in range(12):
        o.step(1)
        dts.append(o.dt())
    # runs at steps 0, 5, 10 (stepModulo); the first keeps dt (nothing may grow yet), later ones grow by
    # (1 + maxRelInc)^5, far below the critical step
    assert dts[0] == 1e-7
    assert all(d == 1e-7 for d in dts[:5])
    assert dts[5] == pytest.approx(1e-7 * 1.001 ** 5, rel=1e-15)
    assert all(d == dts[5] for d in dts[5:10])
    assert dts[10] == pytest.approx(1e-7 * 1.001 ** 10, rel=1e-14)


def test_no_contacts_keeps_dt():
    o, mats, m, kn = _pair(dt=1e-6, period=1)
    # separate the spheres: no real contact -> no critical step, dt unchanged
    o2 = None
    mats_py = [dict(kind=abi.MAT_FRICT, density=2000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    pa = scenes.assemble(np.array([[0.0, 0, 0], [0.5, 0, 0]]), np.array([0.01, 0.01]), 0, [], mats_py)
    p = scenes.default_params(mats, dt=1e-6, gravity=(0, 0, 0), damping=0.0)
    p.dynDtPeriod = 1
    p.dynDtMaxRelInc = 1e-4
    p.dtSafety = 0.9
    o2 = bridge.Oracle(p, pa)
    o2.step(3)
    assert math.isinf(o2.dyndt_crit()) and o2.dt() == 1e-6
