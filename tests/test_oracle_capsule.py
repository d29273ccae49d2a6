"""Known answers of the oracle's capsule functors (src/dem/Capsule.cpp): Cg2_Sphere_Capsule_L6Geom,
Cg2_Wall_Capsule_L6Geom, Cg2_Capsule_Capsule_L6Geom (with CompUtils::distSq_SegmentSegment), and
Capsule::lumpMassInertia.

Capsules of radius 0.02 and shaft 0.1 along the global x axis unless stated; after one step of 1e-9 s
(no gravity) the contact's point, normal (first row of L6Geom.trsf) and uN follow from the geometry:
the closest points of the axis segments, the end caps' overlaps with a wall weighting the contact
point, and for capsules side by side the overlapping ends' points averaged.  The reference's test suite
has no capsule cases, so these pin the restatement."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes

R, SHAFT = 0.02, 0.1
MATS = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]


def quat_z(angle):
    return scenes.quat_from_axis_angle((0, 0, 1), angle)


def capsule_scene(caps, spheres=(), walls=()):
    """caps: [(centre, ori)], spheres: [(centre, radius)], walls: [(axis, sense, position)]."""
    mats = scenes.materials_array(MATS)
    sc = np.array([c for c, _ in spheres], float).reshape(-1, 3)
    sr = np.array([r for _, r in spheres], float)
    pa = scenes.assemble(sc, sr, 0, [(a, s, x, 0) for a, s, x in walls], MATS)
    pa = scenes.add_capsules(pa, [c for c, _ in caps], R, SHAFT, [o for _, o in caps], 0, MATS)
    p = scenes.default_params(mats, dt=1e-9, gravity=(0, 0, 0), damping=0.0)
    return scenes.SceneSpec(p, mats, pa, "caps")


def one_step(spec):
    o = bridge.Oracle(spec.params, spec.particles)
    o.step(1)
    return o.contacts(), o.particles()


def check(c, k, ids, normal, cpt, uN):
    assert (c.idA[k], c.idB[k]) == ids and c.real[k] == 1
    assert np.allclose(c.trsf[k, :3], normal, rtol=0, atol=1e-12)
    assert np.allclose(c.contPt[k], cpt, rtol=0, atol=1e-12)
    assert c.uN[k] == pytest.approx(uN, rel=0, abs=1e-14)


def test_mass_inertia():
    """Capsule::lumpMassInertia: a shaft of 0 is a sphere (inertia 2/5 m r^2 on every axis)."""
    m, I = scenes.capsule_mass_inertia(0.01, 0.0, 2000.0)
    ms = (4 / 3.0) * math.pi * 1e-6 * 2000
    assert m == pytest.approx(ms, rel=1e-15)
    assert np.allclose(I, 0.4 * ms * 1e-4, rtol=1e-14)
    m, I = scenes.capsule_mass_inertia(R, SHAFT, 1000.0)
    assert I[1] == I[2] and I[1] > I[0]


@pytest.mark.parametrize("centre,base", [((.03, .029, 0), (.03, 0, 0)),          # beside the shaft
                                         ((.05 + .02, .0205, 0), (.05, 0, 0)),   # over the end cap
                                         ((-.075, 0, .001), (-.05, 0, 0))])      # beyond the other end
def test_sphere_capsule(centre, base):
    spec = capsule_scene([((0, 0, 0), (1, 0, 0, 0))], spheres=[(centre, 0.01)])
    c, p = one_step(spec)
    assert c.n == 1
    sC, b = np.array(centre), np.array(base)
    dist = np.linalg.norm(b - sC)
    n = (b - sC) / dist
    uN = dist - (0.01 + R)
    check(c, 0, (0, 1), n, sC + n * (0.01 + .5 * uN), uN)


def test_wall_capsule_flat_and_tilted():
    # flat on the wall z = 0: both ends overlap equally, the contact point is the centre's projection
    spec = capsule_scene([((.1, .2, .019), (1, 0, 0, 0))], walls=[(2, 1, 0.0)])
    c, p = one_step(spec)
    check(c, 0, (0, 1), (0, 0, 1), (.1, .2, 0), .019 - R)
    # tilted so that only the lower end overlaps: that end takes all
    q = scenes.quat_from_axis_angle((0, 1, 0), 0.3)
    spec = capsule_scene([((.1, .2, .032), q)], walls=[(2, 1, 0.0)])
    c, p = one_step(spec)
    end = np.array([.1, .2, .032]) + scenes.quat_rotate(q, (SHAFT / 2, 0, 0))
    lower = end if end[2] < .032 else np.array([.1, .2, .032]) - scenes.quat_rotate(q, (SHAFT / 2, 0, 0))
    check(c, 0, (0, 1), (0, 0, 1), (lower[0], lower[1], 0), lower[2] - R)


def test_capsules_crossed():
    """One above the other, perpendicular: the closest points of the axes give everything."""
    spec = capsule_scene([((0, 0, 0), (1, 0, 0, 0)), ((0, 0, .039), quat_z(math.pi / 2))])
    c, p = one_step(spec)
    check(c, 0, (0, 1), (0, 0, 1), (0, 0, R + .5 * (.039 - 2 * R)), .039 - 2 * R)


def test_capsules_side_by_side():
    """Parallel axes (the parallel branch of the segment distance): all four ends overlap, the contact
    point is the mean of the ends' points half-way between the axes."""
    spec = capsule_scene([((0, 0, 0), (1, 0, 0, 0)), ((0, .039, 0), (1, 0, 0, 0))])
    c, p = one_step(spec)
    check(c, 0, (0, 1), (0, 1, 0), (0, .0195, 0), .039 - 2 * R)


def test_capsules_staggered():
    """Parallel and shifted along the axis: one end of each overlaps, the contact point is the middle of
    the overlapping stretch."""
    spec = capsule_scene([((0, 0, 0), (1, 0, 0, 0)), ((.06, .039, 0), (1, 0, 0, 0))])
    c, p = one_step(spec)
    check(c, 0, (0, 1), (0, 1, 0), (.03, .0195, 0), .039 - 2 * R)


def test_segment_regions_match_brute_force():
    """distSq_SegmentSegment through the capsule functor: uN of random capsule pairs against a dense
    sampling of the two segments (all nine regions and the parallel case occur)."""
    rng = np.random.default_rng(5)
    checked = 0
    for _ in range(60):
        c2 = rng.normal(0, .03, 3)
        q1, q2 = scenes.random_quaternions(2, rng)
        if rng.random() < .2:
            q2 = q1  # parallel
        spec = capsule_scene([((0, 0, 0), q1), (tuple(c2), q2)])
        spec.particles.pos[1] = c2
        d1 = scenes.quat_rotate(q1, (1, 0, 0))
        d2 = scenes.quat_rotate(q2, (1, 0, 0))
        t = np.linspace(-SHAFT / 2, SHAFT / 2, 801)
        P = t[:, None] * d1[None, :]
        Q = c2[None, :] + t[:, None] * d2[None, :]
        dmin = np.sqrt(((P[:, None, :] - Q[None, :, :]) ** 2).sum(-1).min())
        if dmin > 2 * R:
            continue
        c, p = one_step(spec)
        real = c.real == 1
        assert real.sum() == 1
        assert c.uN[real][0] == pytest.approx(dmin - 2 * R, abs=2e-4)
        checked += 1
    assert checked > 20
