"""Known answers of the oracle's Cg2_Facet_Sphere_L6Geom (src/dem/Facet.cpp:333-390) and Bo1_Facet_Aabb.

One fixed facet with nodes (0,0,0), (1,0,0), (0,1,0) and one sphere of radius 0.01; after one step of
1e-9 s (no gravity) the contact's point, normal (first row of L6Geom.trsf) and uN follow from the
geometry alone: the sphere's centre projected onto the facet's plane and snapped to the triangle
(interior), to the closest point of an edge, or to a node, then moved by halfThick along the normal.
The reference's test suite has no facet golden vectors (py/tests/test_core.py:95 only builds the
functor), so these cases pin the restatement."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes

R = 0.01
TRI = ((0, 0, 0), (1, 0, 0), (0, 1, 0))


def facet_pair(center, ht=0.0, r=R, tri=TRI, vel=(0, 0, 0)):
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    pa = scenes.assemble(np.array([center], float), np.array([r]), 0, [], mats_py, vel=np.array([vel], float))
    pa = scenes.add_facets(pa, [tri], halfThick=ht)
    p = scenes.default_params(mats, dt=1e-9, gravity=(0, 0, 0), damping=0.0)
    return scenes.SceneSpec(p, mats, pa, "facet_pair")


def one_step(center, **kw):
    spec = facet_pair(center, **kw)
    o = bridge.Oracle(spec.params, spec.particles)
    o.step(1)
    return o.contacts(), o.particles()


CASES = [
    # (sphere centre, halfThick, closest point of the mid-plane triangle, normal) -- w = 0: interior
    ((.3, .3, .0099), 0.0, (.3, .3, 0), (0, 0, 1)),
    ((.3, .3, -.0099), 0.0, (.3, .3, 0), (0, 0, -1)),
    ((.3, .3, .011), .002, (.3, .3, 0), (0, 0, 1)),
    # w = 1, 2, 4: closest point of edge n0-n1, n1-n2, n2-n0
    ((.5, -.005, 0), 0.0, (.5, 0, 0), (0, -1, 0)),
    ((.5 + .004, .5 + .004, 0), 0.0, (.5, .5, 0), (1 / math.sqrt(2), 1 / math.sqrt(2), 0)),
    ((-.005, .5, 0), 0.0, (0, .5, 0), (-1, 0, 0)),
    # w = 5, 3, 6: node 0, node 1, node 2
    ((-.004, -.004, .001), 0.0, (0, 0, 0), None),
    ((1.004, -.003, 0), 0.0, (1, 0, 0), None),
    ((-.003, 1.004, .002), 0.0, (0, 1, 0), None),
]


@pytest.mark.parametrize("center,ht,cpt,normal", CASES)
def test_contact_point_normal_uN(center, ht, cpt, normal):
    c, p = one_step(center, ht=ht)
    assert c.n == 1 and c.real[0] == 1
    # the facet (id 1) is pA, the sphere pB (Cg2_Facet_Sphere_L6Geom takes the facet first)
    assert (c.idA[0], c.idB[0]) == (1, 0)
    sC = np.array(center, float)
    base = np.array(cpt, float)
    if normal is None:
        normal = (sC - base) / np.linalg.norm(sC - base)
    normal = np.array(normal, float)
    assert np.allclose(c.trsf[0, :3], normal, rtol=0, atol=1e-12)
    assert np.allclose(c.contPt[0], base + ht * normal, rtol=0, atol=1e-12)
    assert c.uN[0] == pytest.approx(np.linalg.norm(sC - base) - R - ht, rel=0, abs=1e-15)
    # the sphere is pushed along the normal; the facet receives no force (multi-node shape)
    assert np.dot(p.force[0], normal) > 0
    assert np.array_equal(p.force[1], np.zeros(3))


@pytest.mark.parametrize("center,ht", [((.3, .3, .0101), 0.0), ((.3, .3, .0121), .002), ((-.008, -.008, 0.0), 0.0)])
def test_no_contact_beyond_reach(center, ht):
    """Boxes overlap (the pair is potential) but the functor finds the sphere beyond r + halfThick."""
    c, p = one_step(center, ht=ht)
    assert c.n == 1 and c.real[0] == 0
    assert np.array_equal(p.force[0], np.zeros(3))


def test_kinetic_sphere_bounces_off_facet():
    """A sphere moving into the facet is stopped and sent back (normal force along +z)."""
    spec = facet_pair((.3, .3, .0101), vel=(0, 0, -1.0))
    spec.params.dt = 1e-6
    o = bridge.Oracle(spec.params, spec.particles)
    o.step(2000)
    p = o.particles()
    assert p.vel[0, 2] > 0
    assert np.array_equal(p.pos[1], np.zeros(3))


def test_facet_bounds():
    """Bo1_Facet_Aabb: the nodes +- halfThick, enlarged by verletDist; the collider pairs the sphere whose
    box overlaps the facet's box and not the one whose box does not."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    ht = 0.01
    # sphere 0 above the facet's box by less than its radius + halfThick; sphere 1 far above
    pa = scenes.assemble(np.array([[.2, .2, .015], [.2, .2, .05]]), np.array([R, R]), 0, [], mats_py)
    pa = scenes.add_facets(pa, [TRI], halfThick=ht)
    p = scenes.default_params(mats, dt=1e-9, gravity=(0, 0, 0), damping=0.0, verletDist=0.0)
    o = bridge.Oracle(p, pa)
    o.step(1)
    c = o.contacts()
    assert c.n == 1 and (c.idA[0], c.idB[0]) == (2, 0)
