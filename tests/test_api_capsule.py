"""Capsules through the Woo-like Python surface (no GPU): Capsule.make / utils.capsule construction
(mass and inertia of Capsule::lumpMassInertia), packing into the engine's arrays, defaultEngines' capsule
functors, and a scene stepped on the oracle stand-in of the engine's handle (capsules come to rest lying
on a wall)."""
import numpy as np
import pytest

from woo_gb300 import abi, dem, scenes, utils
from woo_gb300.core import Scene

from oracle_handle import run_on_oracle


def capsule_floor_scene(n=4):
    m = dem.FrictMat(density=2000, young=1e7, ktDivKn=0.2, tanPhi=0.5)
    par = [utils.wall(0, axis=2, sense=1, mat=m)]
    par += [utils.capsule((0.06 * k, 0.0, 0.012 + 0.002 * k), 0.01, 0.03, mat=m) for k in range(n)]
    return Scene(fields=[dem.DemField(gravity=(0, 0, -9.81), par=par)],
                 engines=dem.DemField.minimalEngines(damping=0.5, dynDtPeriod=0), dtSafety=0.5)


def test_capsule_make():
    m = dem.FrictMat(density=1500)
    p = dem.Capsule.make((1, 2, 3), 0.01, 0.04, mat=m)
    mass, inertia = scenes.capsule_mass_inertia(0.01, 0.04, 1500)
    assert p.mass == mass and np.array_equal(p.inertia, inertia)
    assert p.mask == dem.DemField.defaultMovableMask and p.shape.volume() * 1500 == pytest.approx(mass)
    assert np.allclose(p.shape.endPt(1), (1.02, 2, 3))
    with pytest.raises(RuntimeError, match="radius"):
        dem.Capsule.make((0, 0, 0), 0.0, 0.1)


def test_default_engines_have_capsule_functors():
    ee = utils.defaultEngines(dynDtPeriod=0)
    assert any(isinstance(b, dem.Bo1_Capsule_Aabb) for b in ee[1].boundFunctors)
    for cls in (dem.Cg2_Sphere_Capsule_L6Geom, dem.Cg2_Wall_Capsule_L6Geom, dem.Cg2_Capsule_Capsule_L6Geom):
        assert any(isinstance(g, cls) for g in ee[2].geoFunctors)


def test_capsule_packing_and_functors():
    S = capsule_floor_scene()
    S._prepare_dt()
    g = S._engine()
    g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    assert pa.shape[1] == abi.SHAPE_CAPSULE and pa.radius[1] == 0.01 and pa.shaft[1] == 0.03
    assert S.dem.critDt() == pytest.approx(0.01 / np.sqrt(1e7 / 2000))
    S = capsule_floor_scene()
    S.lab.contactLoop.geoFunctors = [dem.Cg2_Sphere_Sphere_L6Geom(), dem.Cg2_Wall_Sphere_L6Geom()]
    with pytest.raises(RuntimeError, match="Cg2_Wall_Capsule_L6Geom"):
        S.run(1)


def test_capsules_rest_on_wall(monkeypatch):
    S = capsule_floor_scene()
    run_on_oracle(monkeypatch, S, 8000)
    for p in S.dem.par:
        if isinstance(p.shape, dem.Capsule):
            assert p.pos[2] == pytest.approx(0.01, abs=2e-4)
            assert np.linalg.norm(p.vel) < 5e-3
    assert {c.id1 for c in S.dem.con} == {0} and len(S.dem.con) == 4
