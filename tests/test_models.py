"""woo.models.ContactModelSelector (py/models.py:212-315) and DemField.minimalEngines(model=...)
(py/utils.py:100-108), on the CPU."""
import warnings

import numpy as np
import pytest

from woo_gb300 import abi, dem, models, utils
from woo_gb300.core import Scene

from oracle_handle import run_on_oracle


def test_functors_and_damping():
    lin = models.ContactModelSelector(name="linear", damping=0.3, linRoll=True, linRollParams=(2., 3., 4.))
    cp2, law = lin.getFunctors()
    assert isinstance(cp2[0], dem.Cp2_FrictMat_FrictPhys) and isinstance(law[0], dem.Law2_L6Geom_FrictPhys_IdealElPl)
    assert (law[0].relRollStiff, law[0].relTwistStiff, law[0].rollTanPhi) == (2., 3., 4.)
    assert lin.getNonviscDamping() == 0.3
    dmt = models.ContactModelSelector(name="DMT", poisson=0.3, restitution=0.7)
    cp2, law = dmt.getFunctors()
    assert isinstance(cp2[0], dem.Cp2_HertzMat_HertzPhys) and (cp2[0].poisson, cp2[0].en) == (0.3, 0.7)
    assert isinstance(law[0], dem.Law2_L6Geom_HertzPhys_DMT)
    assert dmt.getNonviscDamping() == 0.
    for name in ("pellet", "concrete", "ice", "luding"):
        with pytest.raises(ValueError, match="no GPU counterpart"):
            models.ContactModelSelector(name=name)
    with pytest.raises(ValueError, match="Unknown model"):
        models.ContactModelSelector(name="bogus")
    with pytest.raises(ValueError, match="alpha"):
        models.ContactModelSelector(name="DMT", alpha=0.1)


def test_materials_follow_the_model():
    m0 = dem.FrictMat(density=2000, young=3e7, tanPhi=0.4)
    sel = models.ContactModelSelector(name="DMT", numMat=(2, 3), mats=[m0])
    assert len(sel.mats) == 2 and all(type(m) is dem.HertzMat for m in sel.mats)
    assert (sel.mats[0].density, sel.mats[0].young, sel.mats[0].tanPhi) == (2000, 3e7, 0.4)
    sel = models.ContactModelSelector(name="linear", numMat=(1, 1), mats=[dem.FrictMat(), dem.FrictMat()])
    assert len(sel.mats) == 1 and type(sel.mats[0]) is dem.FrictMat


def test_default_engines_with_model():
    sel = models.ContactModelSelector(name="Hertz", restitution=0.8)
    with warnings.catch_warnings(record=True) as w:
        warnings.simplefilter("always")
        ee = utils.defaultEngines(model=sel, damping=0.4, dynDtPeriod=0)
        assert any("damping is ignored" in str(x.message) for x in w)
    assert ee[0].damping == 0.
    assert ee[2].phyFunctors[0].label == "cp2" and ee[2].lawFunctors[0].label == "contactLaw"
    with pytest.raises(ValueError, match="distFactor"):
        utils.defaultEngines(model=models.ContactModelSelector(name="linear", distFactor=1.5))


def _dmt_scene(mat):
    par = [dem.Wall.make(0, axis=2, sense=1, mat=mat)] + \
          [dem.Sphere.make((0.012 * k, 0, 0.006 + 0.0125 * k), 0.006, mat=mat) for k in range(4)]
    sel = models.ContactModelSelector(name="DMT", restitution=0.8)
    return Scene(fields=[dem.DemField(gravity=(0, 0, -9.81), par=par)],
                 engines=dem.DemField.minimalEngines(model=sel, dynDtPeriod=0), dtSafety=0.5)


def test_dmt_scene_runs_with_hertz_materials(monkeypatch):
    sel = models.ContactModelSelector(name="DMT")
    mat = sel.mats[0]
    mat.young, mat.density, mat.surfEnergy = 5e7, 2500., 0.01
    S = _dmt_scene(mat)
    S._prepare_dt()
    p = S._engine()._build_params(S, S.dem)
    assert p.cp2 == abi.CP2_HERTZ and p.law == abi.LAW_HERTZ_DMT and p.en == 0.8
    run_on_oracle(monkeypatch, S, 400)
    assert S.dem.con.countReal() >= 1
    assert np.isfinite(S.dem.par[4].pos).all()


def test_frictmat_with_hertz_cp2_is_refused():
    S = _dmt_scene(dem.FrictMat())
    S._prepare_dt()
    with pytest.raises(RuntimeError, match="needs HertzMat"):
        S._engine()._build_params(S, S.dem)
