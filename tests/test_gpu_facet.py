"""Fixed facets on the GPU (Cg2_Facet_Sphere_L6Geom, Bo1_Facet_Aabb) against the oracle, bit-exact.

- the nine known-answer placements of the oracle's facet test (interior, the three edges, the three
  nodes, both sides, halfThick) after one step: contacts and particles identical;
- 1500 spheres dropped into a V-shaped valley of 60 facets between four walls (8000 steps),
  FrictMat/IdealElPl and HertzMat/DMT, halfThick 0 and 1 mm: particles and contacts identical after every
  block of steps;
- the cases the engine refuses: a facet that is not fixed or moves, facets in a periodic cell, a facet whose
  mask pairs it with a wall (no Cg2_Wall_Facet_L6Geom), non-finite node coordinates;
- the same through the Python surface (Facet.make floor under Scene.run)."""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, dem, scenes

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles
from test_oracle_facet import CASES, facet_pair

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("center,ht,cpt,normal", CASES)
def test_known_placements(wdem_lib, center, ht, cpt, normal):
    spec = facet_pair(center, ht=ht)
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    h.step(1)
    o.step(1)
    cg, co = h.download_contacts(), o.contacts()
    assert cg.n == 1 and cg.real[0] == 1
    assert_same_contacts(cg, co)
    assert np.array_equal(cg.uN, co.uN)
    assert_same_particles(gpu_particles(h, spec.particles.n), o.particles())
    h.close()


def _valley(law, ht, seed):
    spec = scenes.facet_valley(1500, seed, box=(0.25, 0.2, 0.08), law=law, halfThick=ht, vel_scale=0.1)
    nw = 4
    k = spec.info["n_spheres"]
    spec.particles.vel[nw:nw + k, 2] -= 1.5
    return spec


@pytest.mark.parametrize("law,ht", [("frict", 0.0), ("frict", 0.001), ("hertz", 0.0), ("hertz", 0.001)])
def test_valley_bit_exact(wdem_lib, law, ht):
    spec = _valley(law, ht, 7)
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    n = spec.particles.n
    facet = spec.particles.shape == abi.SHAPE_FACET
    seen = 0
    for block in (1, 99, 400, 1500, 3000, 3000):
        h.step(block)
        o.step(block)
        cg, co = h.download_contacts(), o.contacts()
        assert_same_particles(gpu_particles(h, n), o.particles())
        assert_same_contacts(cg, co)
        seen = max(seen, int((cg.real.astype(bool) & facet[cg.idA]).sum()))
    # the spheres reached the facets: real facet contacts were compared
    assert seen >= 50
    pg = gpu_particles(h, n)
    assert np.array_equal(pg.pos[facet], spec.particles.pos[facet])
    h.close()


def _refused(spec, match):
    h = abi.Handle(spec.particles.n)
    h.set_params(spec.params)
    with pytest.raises(abi.WdemError, match=match) as ei:
        h.upload_particles(spec.particles)
        h.step(1)
    h.close()
    return ei.value.code


def test_refusals(wdem_lib):
    spec = facet_pair((.3, .3, .0099))
    spec.particles.flags[1] = 0
    assert _refused(spec, "DOFs blocked") == abi.WDEM_ERR_UNSUPPORTED
    spec = facet_pair((.3, .3, .0099))
    spec.particles.vel[1] = (0, 0, 1e-3)
    assert _refused(spec, "moving facets") == abi.WDEM_ERR_UNSUPPORTED
    spec = facet_pair((.3, .3, .0099))
    spec.particles.facetVerts[1, 4] = np.nan
    assert _refused(spec, "non-finite") == abi.WDEM_ERR_ARG
    # a facet and a wall whose masks meet outside loneMask
    spec = _valley("frict", 0.0, 3)
    spec.params.loneMask = 0
    assert _refused(spec, "wall-facet contacts are not implemented") == abi.WDEM_ERR_UNSUPPORTED


def test_periodic_refused(wdem_lib):
    spec = facet_pair((.3, .3, .0099))
    h = abi.Handle(spec.particles.n)
    h.set_params(spec.params)
    h.set_cell(np.eye(3))
    with pytest.raises(abi.WdemError, match="periodic") as ei:
        h.upload_particles(spec.particles)
    assert ei.value.code == abi.WDEM_ERR_UNSUPPORTED
    h.close()


def test_scene_api(wdem_lib):
    """The Python surface (Facet.make floor, spheres, minimalEngines) on the GPU: the spheres' trajectories
    equal the oracle's bit for bit."""
    from test_api_facet import facet_floor_scene
    S = facet_floor_scene(ht=0.002)
    S._prepare_dt()
    g = S._engine()
    params = g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    o = bridge.Oracle(params, pa)
    S.run(3000)
    o.step(3000)
    po = o.particles()
    for p in S.dem.par:
        if isinstance(p.shape, dem.Sphere):
            assert np.array_equal(p.pos, po.pos[p.id]) and np.array_equal(p.vel, po.vel[p.id])
    assert len(S.dem.con) == o.contacts().n
