"""Periodic cell in the oracle: the known answers of py/tests/test_pbc.py (incident velocity across 10
cells with homoDeform gradV2, the cell's trsf/hSize recursion, over-half-cell contacts, the
double-contact error, cellDist of shifted spheres, a pair formed across the boundary) and the periodic pair predicate against brute force
over images."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, scenes


def test_l6geom_incident_velocity_gradv2():
    """py/tests/test_pbc.py:86-95 (testL6GeomIncidentVelocity): sphere #1 ten cells away along z moving at
    5 m/s; with nextGradV = diag(0,0,-1) its absolute velocity picks up the mean field, and the contact's
    incident velocity, corrected by Cell.intrShiftVel, is the initial 5 m/s again."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7, ktDivKn=0.2, tanPhi=math.tan(0.5))]
    mats = scenes.materials_array(mats_py)
    init_pos = np.array([1.0, 1.0 + 1.0, 1.0 + 10 * 3.0])
    pa = scenes.assemble(np.array([[1.0, 1, 1], init_pos]), np.array([0.5, 0.5]), 0, [], mats_py,
                         vel=np.array([[0, 0, 0], [0, 0, 5.0]]))
    p = scenes.default_params(mats, dt=0.0, damping=0.0, noBreak=1)
    o = bridge.Oracle(p, pa, cell=dict(hSize=np.diag([2.5, 2.5, 3.0]), nextGradV=np.diag([0, 0, -1.0])))
    o.step(1)                      # dt=0: only the velocity gradient takes effect
    v = o.particles().vel
    assert v[1, 2] == pytest.approx(5.0 - 31.0) and v[0, 2] == pytest.approx(-1.0)
    p.dt = 1e-10
    p.step = 1
    o.lib.orc_set_params(o.h, __import__("ctypes").byref(p))
    o.step(1)
    c = o.contacts()
    assert c.n == 1 and c.real[0] == 1
    assert np.array_equal(c.cellDist[0], [0, 0, -10])
    assert np.linalg.norm(c.geomVel[0]) == pytest.approx(np.linalg.norm([0, 0, 5.0]), abs=1e-7)



def test_cell_integration_gradv2():
    """py/tests/test_pbc.py:35-50 (testVelGrad) in the homoDeform mode restated here (gradV2): each step,
    Cell::integrateAndUpdate (src/core/Cell.cpp:81-100) accumulates trsf += dt gradV trsf, the recursion
    the reference's test checks, and advances hSize by the midpoint rule
    hSize = (I - gradV dt/2)^-1 (I + gradV dt/2) hSize (the gradV2 branch; the test's own
    hSize += dt gradV hSize is the other modes' first-order rule), with pprevHsize the mean of the old
    and the new hSize.  A simple shear with a compression, over 10 steps."""
    G = np.array([[0.0, 0.4, 0.0], [0.0, 0.0, 0.0], [0.0, 0.0, -1.0]])
    dt = 1e-3
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7)]
    mats = scenes.materials_array(mats_py)
    pa = scenes.assemble(np.array([[1.0, 1.0, 1.0]]), np.array([0.1]), 0, [], mats_py)
    p = scenes.default_params(mats, dt=dt, damping=0.0)
    h0 = np.diag([2.5, 2.5, 3.0])
    o = bridge.Oracle(p, pa, cell=dict(hSize=h0, gradV=G, nextGradV=G))
    eye = np.eye(3)
    hs, tr, first = h0.copy(), eye.copy(), h0.copy()
    for _ in range(10):
        prev = hs
        tr = tr + dt * G @ tr
        hs = np.linalg.solve(eye - G * dt / 2, (eye + G * dt / 2) @ hs)
        first = first + dt * G @ first
        o.step(1)
        c = o.cell()
        np.testing.assert_allclose(c["trsf"], tr, rtol=0, atol=1e-14)
        np.testing.assert_allclose(c["hSize"], hs, rtol=0, atol=3e-14)
        np.testing.assert_allclose(c["pprevHsize"], (prev + hs) / 2, rtol=0, atol=3e-14)
    # the midpoint rule and the first-order one part at O(dt^2) per step: the two modes are distinct
    assert abs(c["hSize"][2, 2] - first[2, 2]) > 1e-6
    assert c["hSize"][2, 2] == pytest.approx(3.0 * ((1 - dt / 2) / (1 + dt / 2)) ** 10, rel=1e-14)

def _image_pairs(pos, r, size):
    """Brute force over all pairs: the integer cell shift k (per axis) of box 2 for which the boxes
    overlap strictly, as spatialOverlapPeri requires; boxes are smaller than half the cell, so at most
    one k per axis exists."""
    n = len(r)
    i, j = np.triu_indices(n, 1)
    mn, mx = pos - r[:, None], pos + r[:, None]
    lo = (mn[i] - mx[j]) / size          # k*size must lie in (mn1-mx2, mx1-mn2)
    hi = (mx[i] - mn[j]) / size
    k = np.floor(lo) + 1
    ok = np.all((k * size > mn[i] - mx[j]) & (k * size < mx[i] - mn[j]), axis=1)
    return {(int(a), int(b)): tuple(int(v) for v in kk) for a, b, kk in zip(i[ok], j[ok], k[ok])}


def test_periodic_pairs_match_images():
    """The oracle's periodic pair set (cell list + spatialOverlapPeri) equals the brute-force set of
    pairs whose boxes overlap for some periodic image, with Contact.cellDist = that image."""
    rng = np.random.default_rng(3)
    n = 250
    size = np.array([0.2, 0.25, 0.3])
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7)]
    mats = scenes.materials_array(mats_py)
    pos = rng.uniform(-0.3, 0.6, (n, 3))     # positions are not wrapped into the cell
    r = rng.uniform(0.006, 0.014, n)
    pa = scenes.assemble(pos, r, 0, [], mats_py)
    p = scenes.default_params(mats, dt=1e-9, damping=0.0, verletDist=0.0)
    o = bridge.Oracle(p, pa, cell=dict(hSize=np.diag(size)))
    o.step(1)
    c = o.contacts()
    got = {(int(a), int(b)): tuple(int(v) for v in d) for a, b, d in zip(c.idA, c.idB, c.cellDist)}
    exp = _image_pairs(pos, r, size)
    assert len(exp) > 50
    assert got == exp


def _two_spheres(c0, r0, c1, r1):
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    pa = scenes.assemble(np.array([c0, c1], float), np.array([r0, r1]), 0, [], mats_py)
    p = scenes.default_params(mats, dt=1e-8, gravity=(0, 0, 0), damping=0.0)
    return bridge.Oracle(p, pa, cell=dict(hSize=np.eye(3))), mats


@pytest.mark.parametrize("shift", [(0, 0, 0), (13, 14, 15)])
def test_over_half_cell_contact(shift):
    """py/tests/test_pbc.py:130-144 (testOverHalfContact): a sphere spanning more than half the unit cell;
    the pair's cellDist follows a shift of the first sphere by whole cells."""
    o, _ = _two_spheres(np.array([.3, .5, .5]) + shift, .4, (.7, .9, .5), .1)
    o.step(1)
    c = o.contacts()
    assert c.n == 1 and (c.idA[0], c.idB[0]) == (0, 1)
    assert tuple(c.cellDist[0]) == shift


def test_double_contact_is_an_error():
    """py/tests/test_pbc.py:145-155 (testDoubleContact): boxes overlapping on both sides across the cell
    are an error of the collider."""
    o, _ = _two_spheres((.3, .5, .5), .4, (.8, .9, .5), .2)
    with pytest.raises(RuntimeError, match="ambiguous periodic contact"):
        o.step(1)


@pytest.mark.parametrize("shift", [(0, 0, 0), (1, 2, 3), (6, 8, -4)])
def test_normal_contact_cell_dist(shift):
    """py/tests/test_pbc.py:156-169 (testNormalContact): a real contact whose second sphere is moved by
    whole cells has cellDist = -shift."""
    o, _ = _two_spheres((.5, .5, .5), .2, np.array([.8, .6, .5]) + shift, .2)
    o.step(1)
    c = o.contacts()
    assert c.n == 1 and c.real[0] == 1
    assert tuple(c.cellDist[0]) == tuple(-np.array(shift))


def test_cross_boundary_pair():
    """py/tests/test_pbc.py:174-203 (testCrossBoundarySort) in its observable form: with verletDist 0 the
    collider runs every step; a sphere that crosses the cell's x boundary in its second step, from the
    incrementally sorted state of the first, is paired with the sphere near x = 0 through the next
    period (cellDist -1 on x, the pair set of the brute-force image search), and not before."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    r = 0.02
    pos = np.array([[0.02, 0.5, 0.5], [0.52, 0.5, 0.5], [0.8, 0.2, 0.2]])
    pa = scenes.assemble(pos, np.full(3, r), 0, [], mats_py, vel=np.array([[0, 0, 0], [0.265, 0, 0], [0, 0, 0]]))
    p = scenes.default_params(mats, dt=1.0, damping=0.0, verletDist=0.0)
    o = bridge.Oracle(p, pa, cell=dict(hSize=np.eye(3)))
    o.step(1)                                   # sphere 1 at x = 0.785: no pair
    assert o.contacts().n == 0
    o.step(1)                                   # x = 1.05, i.e. 0.05 in the next period: overlaps sphere 0
    x = o.particles().pos
    assert x[1, 0] == pytest.approx(1.05)
    c = o.contacts()
    got = {(int(a), int(b)): tuple(int(v) for v in d) for a, b, d in zip(c.idA, c.idB, c.cellDist)}
    assert got == {(0, 1): (-1, 0, 0)} == _image_pairs(x, np.full(3, r), np.ones(3))
    assert c.real[0] == 1


def test_stress_of_one_contact_across_the_boundary():
    """ContactLoop's stress (src/dem/ContactLoop.cpp:218-229, 244): the sum over real contacts of the global
    contact force times the branch vector (from A to B through the contact's period), over the cell
    volume.  One FrictPhys pair of equal spheres meeting across the x boundary of a 1 x 1 x 1 cell, at
    rest, with overlap d: kn = E A / (l0 + l1) with A = pi r^2 and l0 = l1 = r (Cp2_FrictMat_FrictPhys,
    src/dem/FrictMat.cpp:39), the normal force kn uN along the normal from A to B, so
    stress_xx = kn uN |branch| / V (negative: compression), every other component zero."""
    r, E = 0.05, 1e7
    mats_py = [dict(kind=abi.MAT_FRICT, density=1000.0, young=E, ktDivKn=0.2, tanPhi=0.5)]
    mats = scenes.materials_array(mats_py)
    pos = np.array([[0.05, 0.5, 0.5], [0.96, 0.5, 0.5]])   # B's image at x = -0.04: centre distance 0.09
    pa = scenes.assemble(pos, np.array([r, r]), 0, [], mats_py)
    p = scenes.default_params(mats, dt=1e-9, damping=0.0)
    o = bridge.Oracle(p, pa, cell=dict(hSize=np.eye(3)))
    o.step(1)
    c = o.contacts()
    assert c.n == 1 and c.real[0] == 1 and tuple(c.cellDist[0]) == (-1, 0, 0)
    un = c.uN[0]
    assert un == pytest.approx(-0.01, rel=1e-12)
    kn = E * math.pi * r * r / (2 * r)
    assert c.kn[0] == pytest.approx(kn, rel=1e-14)
    s = o.stress()
    assert s[0, 0] == pytest.approx(kn * un * 0.09, rel=1e-12)
    off = s.copy()
    off[0, 0] = 0.0
    assert np.all(off == 0.0)
