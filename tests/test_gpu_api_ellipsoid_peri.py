"""Ellipsoids and periodic cells scripted through the Woo-style Python surface, on the GPU, against the
oracle: py/tests/test_ellipsoid.py:24-57 (two ellipsoids touching, rotated, at five scales) and a
sheared periodic packing built with Scene.periodic / Cell.setBox / Cell.nextGradV."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, dem, scenes, utils
from woo_gb300.core import Scene

pytestmark = pytest.mark.gpu


def _ell_engines(**geo):
    return [dem.Leapfrog(reset=True, damping=.4), dem.InsertionSortCollider([dem.Bo1_Ellipsoid_Aabb()], verletDist=0.),
            dem.ContactLoop([dem.Cg2_Ellipsoid_Ellipsoid_L6Geom(**geo)], [dem.Cp2_FrictMat_FrictPhys()],
                            [dem.Law2_L6Geom_FrictPhys_IdealElPl(noBreak=True)])]


def _oracle_for(S):
    S._prepare_dt()
    g = S._engine()
    params = g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    cell = None
    if S.periodic:
        cell = dict(hSize=S.cell.hSize, trsf=S.cell.trsf, gradV=S.cell.gradV, nextGradV=S.cell.nextGradV)
    return bridge.Oracle(params, pa, cell=cell)


@pytest.mark.parametrize("scale", [.5 / 3., 1. / 3., 10. / 3., 100. / 3., 1000 / 3.])
@pytest.mark.parametrize("brent", [True, False])
def test_normal_displacement_ellipsoid_script(wdem_lib, scale, brent):
    mat = dem.FrictMat(density=1e3, young=1e8, ktDivKn=.2, tanPhi=.5)
    gOri = scenes.quat_from_axis_angle(np.array([.1, 1, .3]), math.pi / 3.)
    S = Scene(fields=[dem.DemField()], engines=_ell_engines(brent=brent), dtSafety=.7)
    S.dem.par.add([dem.Ellipsoid.make((0, 0, 0), semiAxes=scale * np.array([.1, .2, .1]), ori=gOri, mat=mat, fixed=True),
                   dem.Ellipsoid.make(scenes.quat_rotate(gOri, scale * np.array([.3, 0, 0])),
                                      semiAxes=scale * np.array([.2, .1, .1]), ori=gOri, mat=mat, fixed=True)], nodes=True)
    S.dem.par[1].vel = scenes.quat_rotate(gOri, np.array([-.1, 0, 0]))
    S.dt = .1
    o = _oracle_for(S)
    S.one()
    o.step(1)
    C = S.dem.con[0]
    # e1 moves by -.1 x .1 = .01 towards e0: that is the overlap
    assert C.geom.uN == pytest.approx(-.01, abs=1e-5 * .01)
    co = o.contacts()
    if brent:
        assert C.geom.uN == co.uN[0]
        assert np.array_equal(C.phys.force, co.force[0])
    else:
        assert C.geom.uN == pytest.approx(co.uN[0], abs=1e-9 * scale)
    assert S.dem.par[0].mass == pytest.approx(1e3 * 4 / 3. * math.pi * .002 * scale ** 3)


def _peri_scene(shear):
    rng = np.random.default_rng(5)
    m = dem.FrictMat(density=1e3, young=1e6, ktDivKn=.2, tanPhi=.4)
    S = Scene(fields=[dem.DemField(gravity=(0, 0, 0))], engines=utils.defaultEngines(damping=.2, dynDtPeriod=0), dtSafety=.5)
    S.periodic = True
    S.cell.setBox(4, 4, 4)
    S.cell.nextGradV = np.array([[0, 0, shear], [0, 0, 0], [0, 0, 0]])
    for ix in range(4):
        for iy in range(4):
            for iz in range(4):
                c = np.array([ix, iy, iz]) + .5 + rng.uniform(-.05, .05, 3)
                S.dem.par.add(utils.sphere(c, .49 + .02 * rng.random(), mat=m, vel=rng.normal(0, .3, 3)))
    return S


@pytest.mark.parametrize("shear", [0.0, 0.2])
def test_periodic_shear_script(wdem_lib, shear):
    S = _peri_scene(shear)
    o = _oracle_for(S)
    for chunk in (1, 49, 150):
        S.run(chunk)
        o.step(chunk)
        po = o.particles()
        pos = np.array([p.pos for p in S.dem.par])
        vel = np.array([p.vel for p in S.dem.par])
        assert np.array_equal(pos, po.pos), "positions differ"
        assert np.array_equal(vel, po.vel), "velocities differ"
        oc = o.cell()
        assert np.array_equal(S.cell.hSize, oc["hSize"]) and np.array_equal(S.cell.trsf, oc["trsf"])
    oc = o.contacts()
    assert len(S.dem.con) == oc.n
    assert S.dem.con.countReal() == int(np.count_nonzero(oc.real)) > 0
    if shear:
        assert 0 < S.cell.hSize[0, 2] <= 200 * S.dt * shear * 4 * (1 + 1e-12)
        assert np.array_equal(S.cell.gradV, S.cell.nextGradV)
