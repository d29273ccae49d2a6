"""Facets through the Woo-like Python surface (no GPU): Facet.make / utils.facet construction, packing into
the engine's arrays, defaultEngines' facet functors, and a scene stepped on the oracle stand-in of the
engine's handle (spheres come to rest on a floor of two facets)."""
import numpy as np
import pytest

from woo_gb300 import abi, dem, utils
from woo_gb300.core import Scene

from oracle_handle import run_on_oracle

FLOOR = [((0, 0, 0), (1, 0, 0), (1, 1, 0)), ((0, 0, 0), (1, 1, 0), (0, 1, 0))]


def facet_floor_scene(n=5, ht=0.0):
    m = dem.FrictMat(density=2500, young=1e7, ktDivKn=0.2, tanPhi=0.5)
    par = [utils.facet(v, halfThick=ht, mat=m) for v in FLOOR]
    par += [dem.Sphere.make((0.2 + 0.15 * k, 0.3 + 0.1 * k, 0.02 + ht), 0.01, mat=m) for k in range(n)]
    return Scene(fields=[dem.DemField(gravity=(0, 0, -9.81), par=par)],
                 engines=dem.DemField.minimalEngines(damping=0.4, dynDtPeriod=0), dtSafety=0.5)


def test_facet_make():
    f = dem.Facet.make(FLOOR[0], halfThick=0.001)
    assert isinstance(f.shape, dem.Facet) and len(f.shape.nodes) == 3
    assert f.mask == dem.DemField.defaultBoundaryMask
    assert all(nd.dem.blocked == "xyzXYZ" and nd.dem.mass == 0 for nd in f.shape.nodes)
    assert np.allclose(f.shape.getNormal(), (0, 0, 1))
    assert f.shape.getArea() == pytest.approx(0.5)
    with pytest.raises(RuntimeError, match="uninodal"):
        f.pos
    with pytest.raises(RuntimeError, match="fakeVel"):
        dem.Facet.make(FLOOR[0], fakeVel=(1, 0, 0))


def test_default_engines_have_facet_functors():
    ee = utils.defaultEngines(dynDtPeriod=0)
    assert any(isinstance(b, dem.Bo1_Facet_Aabb) for b in ee[1].boundFunctors)
    assert any(isinstance(g, dem.Cg2_Facet_Sphere_L6Geom) for g in ee[2].geoFunctors)


def test_facet_packing():
    S = facet_floor_scene(ht=0.002)
    S._prepare_dt()
    g = S._engine()
    g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    assert list(pa.shape[:2]) == [abi.SHAPE_FACET] * 2 and pa.radius[0] == 0.002
    assert np.array_equal(pa.facetVerts[1].reshape(3, 3), np.array(FLOOR[1], float))
    assert np.array_equal(pa.pos[1], FLOOR[1][0]) and pa.flags[0] == 63 and pa.mass[0] == 0


def test_facet_needs_its_functor():
    S = facet_floor_scene()
    S.lab.contactLoop.geoFunctors = [dem.Cg2_Sphere_Sphere_L6Geom(), dem.Cg2_Wall_Sphere_L6Geom()]
    with pytest.raises(RuntimeError, match="Cg2_Facet_Sphere_L6Geom"):
        S.run(1)


@pytest.mark.parametrize("ht", [0.0, 0.002])
def test_spheres_rest_on_facets(monkeypatch, ht):
    S = facet_floor_scene(ht=ht)
    run_on_oracle(monkeypatch, S, 6000)
    for p in S.dem.par:
        if isinstance(p.shape, dem.Sphere):
            assert p.pos[2] == pytest.approx(0.01 + ht, abs=2e-4)
            assert abs(p.vel[2]) < 1e-2
    real = [c for c in S.dem.con if c.real]
    # every sphere rests on a facet (the facet is pA); sphere #4 lies on the shared diagonal edge and touches both
    assert {c.id2 for c in real} == set(range(2, 7)) and all(c.id1 in (0, 1) for c in real)
    assert sorted(c.id1 for c in real if c.id2 == 4) == [0, 1]
    assert np.array_equal(S.dem.par[0].shape.nodes[1].pos, FLOOR[0][1])
