"""Ellipsoids and the periodic cell through the Woo-style Python surface, without a GPU: the shape's mass
and inertia (py/tests/test_ellipsoid.py:63-72), functor attributes packed into wdem_params, the cell's
setBox / degenerate-cell error (py/tests/test_pbc.py:56-66) and the rejection of what the engine does not do."""
import math

import numpy as np
import pytest

from woo_gb300 import abi, dem, utils
from woo_gb300.core import Cell, Scene


def _ell_engines(**geo):
    return [dem.Leapfrog(reset=True, damping=.4), dem.InsertionSortCollider([dem.Bo1_Ellipsoid_Aabb()], verletDist=0.),
            dem.ContactLoop([dem.Cg2_Ellipsoid_Ellipsoid_L6Geom(**geo)], [dem.Cp2_FrictMat_FrictPhys()],
                            [dem.Law2_L6Geom_FrictPhys_IdealElPl(noBreak=True)])]


def test_ellipsoid_mass_inertia():
    a, b, c, rho = 1, 2, 3, 1
    e = dem.Ellipsoid.make(center=(0, 0, 0), semiAxes=(a, b, c), mat=dem.FrictMat(density=rho))
    m = rho * (4 / 3.) * math.pi * a * b * c
    inertia = (1 / 5.) * m * np.array([b ** 2 + c ** 2, a ** 2 + c ** 2, a ** 2 + b ** 2])
    assert e.mass == pytest.approx(m, rel=1e-14)
    assert np.allclose(e.inertia, inertia, rtol=1e-14)
    assert e.shape.equivRadius() == pytest.approx(6 ** (1 / 3.))
    with pytest.raises(RuntimeError):
        dem.Ellipsoid.make((0, 0, 0), semiAxes=(1, 0, 1))


@pytest.mark.parametrize("geo,solver,warm", [({}, abi.ELL_BRENT, abi.WARM_COLD),
                                             (dict(brent=False, warmStart="history", newtonTol=1e-9), abi.ELL_NEWTON, abi.WARM_HISTORY)])
def test_ellipsoid_params_packing(geo, solver, warm):
    mat = dem.FrictMat(density=1e3, young=1e8, ktDivKn=.2, tanPhi=.5)
    S = Scene(fields=[dem.DemField(par=[dem.Ellipsoid.make((0, 0, 0), (.1, .2, .1), mat=mat),
                                        dem.Ellipsoid.make((.3, 0, 0), (.2, .1, .1), mat=mat)])],
              engines=_ell_engines(**geo), dtSafety=.7)
    S._prepare_dt()
    g = S._engine()
    p = g._build_params(S, S.dem)
    assert p.ellSolver == solver and p.warmStart == warm and p.brentBits == 32
    assert p.newtonTol == geo.get("newtonTol", 1e-10)
    pa = g._pack(S.dem)
    assert list(pa.shape) == [abi.SHAPE_ELLIPSOID] * 2
    assert np.array_equal(pa.semiAxes, [[.1, .2, .1], [.2, .1, .1]])
    assert np.all(np.isnan(pa.angMom))
    # critDt: smallest semi-axis over the p-wave speed, times dtSafety
    assert S.dt == pytest.approx(.7 * .1 / math.sqrt(1e8 / 1e3))


def test_ellipsoids_need_their_functor():
    S = Scene(fields=[dem.DemField(par=[dem.Ellipsoid.make((0, 0, 0), (.1, .2, .1))])],
              engines=utils.defaultEngines(dynDtPeriod=0), dt=1e-5)
    g = S._engine()
    with pytest.raises(RuntimeError, match="Cg2_Ellipsoid_Ellipsoid_L6Geom"):
        g._build_params(S, S.dem)


def test_mlp_warm_start_needs_weights():
    S = Scene(fields=[dem.DemField(par=[dem.Ellipsoid.make((0, 0, 0), (.1, .2, .1))])],
              engines=_ell_engines(brent=False, warmStart="mlp"), dt=1e-5)
    g = S._engine()
    assert g._build_params(S, S.dem).warmStart == abi.WARM_MLP


def test_cell_setbox_and_degenerate():
    S = Scene(fields=[dem.DemField()])
    assert S.periodic is False
    S.periodic = True
    S.cell.setBox(2.55, 11, 45)
    assert np.array_equal(S.cell.hSize, np.diag([2.55, 11, 45]))
    S.cell.setBox((1, 2, 3))
    assert S.cell.volume == pytest.approx(6.0)
    assert np.array_equal(S.cell.size, [1, 2, 3])
    with pytest.raises(RuntimeError):
        S.cell.hSize = np.array([[1, 0, 0], [0, 0, 0], [0, 0, 1]])
    assert np.array_equal(S.cell.hSize0, S.cell.hSize)


def test_cell_only_gradv2():
    c = Cell()
    assert c.homoDeform == "gradV2"
    c.homoDeform = 4
    for mode in ("pos", "vel", "vel2", "none"):
        with pytest.raises(RuntimeError):
            c.homoDeform = mode
    with pytest.raises(ValueError):
        c.homoDeform = "bogus"


def test_utils_ellipsoid():
    """woo.utils.ellipsoid (py/utils.py:201-211) gives the same particle as Ellipsoid.make."""
    from woo_gb300 import utils as U
    a = U.ellipsoid((1, 2, 3), (0.1, 0.2, 0.3), ori=(0, 1, 0, 0), angVel=(0, 0, 2))
    b = dem.Ellipsoid.make((1, 2, 3), (0.1, 0.2, 0.3), ori=(0, 1, 0, 0))
    assert a.mass == b.mass and np.array_equal(a.inertia, b.inertia) and np.array_equal(a.ori, b.ori)
    assert np.array_equal(a.angVel, [0, 0, 2]) and a.mask == dem.DemField.defaultMovableMask
