"""Inlets (src/dem/Inlet.cpp) through the Python surface on the CPU, with the engine's handle on the
oracle: mass-rate bookkeeping, non-overlapping placement, the maxNum / maxMass / maxAttempts endings,
reuse of removed ids, and growth of the engine past its capacity."""
import math

import numpy as np
import pytest

from woo_gb300 import dem
from woo_gb300.core import Scene

from oracle_handle import run_on_oracle


def bin_scene(engines=(), gravity=(0, 0, -9.81), n_pre=0, **kw):
    """A 10 x 10 cm walled bin with a floor; n_pre spheres of radius 6 mm already in it."""
    m = dem.FrictMat(density=2500, young=1e7, ktDivKn=0.2, tanPhi=0.5)
    par = [dem.Wall.make(-0.05, axis=0, sense=1, mat=m), dem.Wall.make(0.05, axis=0, sense=-1, mat=m),
           dem.Wall.make(-0.05, axis=1, sense=1, mat=m), dem.Wall.make(0.05, axis=1, sense=-1, mat=m),
           dem.Wall.make(0, axis=2, sense=1, mat=m)]
    for k in range(n_pre):
        par.append(dem.Sphere.make((-0.03 + 0.015 * (k % 5), -0.03 + 0.015 * (k // 5 % 5), 0.006 + 0.013 * (k // 25)),
                                   0.006, mat=m))
    S = Scene(fields=[dem.DemField(gravity=gravity, par=par)],
              engines=dem.DemField.minimalEngines(damping=0.2, dynDtPeriod=0) + list(engines), dtSafety=0.9, **kw)
    return S, m


def inlet(mat, **kw):
    kw.setdefault("box", ((-0.05, -0.05, 0.1), (0.05, 0.05, 0.2)))
    kw.setdefault("stepPeriod", 100)
    return dem.BoxInlet(materials=[mat], generator=dem.MinMaxSphereGenerator(dRange=(0.008, 0.012)), **kw)


def _no_overlap(S, ids):
    c = np.array([S.dem.par[i].pos for i in ids])
    r = np.array([S.dem.par[i].shape.radius for i in ids])
    d = np.sqrt(((c[:, None, :] - c[None, :, :]) ** 2).sum(-1))
    np.fill_diagonal(d, np.inf)
    return bool((d >= r[:, None] + r[None, :]).all())


def test_mass_rate_bookkeeping(monkeypatch):
    S, m = bin_scene(gravity=(0, 0, 0))
    ii = inlet(m, massRate=0.2, seed=3)
    S.engines = S.engines + [ii]
    n0 = len(S.dem.par)
    run_on_oracle(monkeypatch, S, 701)                    # runs at steps 0, 100, ..., 700
    assert ii.nDone == 8
    # the first run sees no elapsed steps (stepPrev is this step, Inlet.cpp:251-254): goal grows 7 times
    goal = 0.2 * S.dt * 700
    assert ii.stepGoalMass == pytest.approx(goal, rel=1e-12)
    assert goal <= ii.mass < goal + 2500 * 4 / 3 * math.pi * 0.006 ** 3
    new = list(range(n0, len(S.dem.par)))
    assert ii.num == len(new) > 5
    assert ii.mass == pytest.approx(sum(S.dem.par[i].mass for i in new), rel=1e-12)
    assert all(S.dem.par[i].mask == dem.DemField.defaultInletMask for i in new)
    # zero gravity and no velocity: placed without overlap, the spheres stay where they were put
    assert _no_overlap(S, new)
    lo, hi = np.array([-0.05, -0.05, 0.1]), np.array([0.05, 0.05, 0.2])
    for i in new:
        p, r = S.dem.par[i].pos, S.dem.par[i].shape.radius
        assert np.all(p - r >= lo) and np.all(p + r <= hi)
        assert 0.004 <= r <= 0.006
    assert S.dem.con.countReal() == 0
    d, mm = ii.generator.diamMass()
    assert len(d) == ii.num and mm.sum() == pytest.approx(ii.mass, rel=1e-12)
    assert math.isfinite(ii.currRate) and ii.currRate > 0


def test_max_num_ends_and_particles_fall(monkeypatch):
    S, m = bin_scene()
    ii = inlet(m, massRate=5.0, maxNum=12, seed=1)
    S.engines = S.engines + [ii]
    n0 = len(S.dem.par)
    run_on_oracle(monkeypatch, S, 2001)
    assert ii.num == 12 and ii.dead and ii.currRate == 0.
    assert len(S.dem.par) == n0 + 12
    zs = [S.dem.par[i].pos[2] for i in range(n0, n0 + 12)]
    assert max(zs) < 0.1                                  # fell out of the inlet box, bouncing on the floor
    assert min(S.dem.par[i].pos[2] - S.dem.par[i].shape.radius for i in range(n0, n0 + 12)) > -0.002


def test_fill_until_attempts_fail(monkeypatch):
    """massRate=0: as many particles as fit (maxAttempts failures end the run, Inlet.cpp:306-311)."""
    S, m = bin_scene(gravity=(0, 0, 0))
    ii = inlet(m, massRate=0, maxAttempts=300, seed=2, box=((-0.02, -0.02, 0.1), (0.02, 0.02, 0.14)))
    S.engines = S.engines + [ii]
    run_on_oracle(monkeypatch, S, 1)
    assert 15 <= ii.num <= 64
    new = list(range(5, len(S.dem.par)))
    assert _no_overlap(S, new)


def test_max_attempts_error_and_dead(monkeypatch):
    S, m = bin_scene(gravity=(0, 0, 0))
    tiny = ((-0.003, -0.003, 0.1), (0.003, 0.003, 0.106))  # smaller than every generated sphere
    ii = inlet(m, massRate=1.0, maxAttempts=50, box=tiny)
    S.engines = S.engines + [ii]
    with pytest.raises(RuntimeError, match="maxAttempts reached"):
        run_on_oracle(monkeypatch, S, 101)
    S2, m2 = bin_scene(gravity=(0, 0, 0))
    ij = inlet(m2, massRate=1.0, maxAttempts=50, box=tiny, atMaxAttempts="dead")
    S2.engines = S2.engines + [ij]
    run_on_oracle(monkeypatch, S2, 201)
    assert ij.dead and ij.num == 0


def test_removed_ids_are_reused(monkeypatch):
    S, m = bin_scene(n_pre=10, gravity=(0, 0, 0))
    S.dem.par[7].pos = (0.0, 0.0, -0.5)                   # below the floor: the outlet takes them
    S.dem.par[9].pos = (0.01, 0.0, -0.5)
    out = dem.BoxOutlet(box=((-1, -1, -0.1), (1, 1, 1)), stepPeriod=50)
    ii = inlet(m, massRate=0.5, maxNum=3, seed=4, stepPeriod=100)
    S.engines = S.engines + [out, ii]
    n0 = len(S.dem.par)
    run_on_oracle(monkeypatch, S, 201)
    assert out.num == 2 and ii.num == 3
    # ParticleContainer::findFreeId: the freed ids first (in the order they were freed), then the end
    assert len(S.dem.par) == n0 + 1
    assert all(S.dem.par.exists(i) for i in range(n0 + 1))
    assert S.dem.par[7].mask == S.dem.par[9].mask == S.dem.par[n0].mask == dem.DemField.defaultInletMask


def test_growth_past_capacity_keeps_state(monkeypatch):
    """More particles than the engine has room for: a new handle takes the state over; accumulated
    energies continue, and the scene matches one run with room to spare from the start."""
    runs = []
    for cap in (0, 1):
        S, m = bin_scene(n_pre=20, trackEnergy=True)
        ii = inlet(m, massRate=1.0, maxNum=30, seed=6,
                   shooter=dem.AlignedMinMaxShooter(dir=(0, 0, -1), vRange=(0.1, 0.5)))
        S.engines = S.engines + [ii]
        S._engine().capacity = (len(S.dem.par) + 1) if cap else 0
        run_on_oracle(monkeypatch, S, 1501)
        runs.append(S)
    a, b = runs
    assert a._gpu._cap >= len(a.dem.par) and len(b.dem.par) <= b._gpu._cap < 2 * len(b.dem.par)
    assert b._gpu._cap > 26                               # the small-capacity run went through a new handle
    assert len(a.dem.par) == len(b.dem.par)
    for i in range(len(a.dem.par)):
        assert np.array_equal(a.dem.par[i].pos, b.dem.par[i].pos)
    ea, eb = a.energy, b.energy
    assert ea["kinInlet"] < 0                             # -Ek of the shot particles (Inlet.cpp:484)
    for k in ("grav", "nonviscDamp", "kinInlet"):
        assert eb[k] == pytest.approx(ea[k], rel=1e-12), k
    assert eb["kinetic"] == pytest.approx(ea["kinetic"], rel=1e-12)


def test_inlet_crit_dt_and_rejections():
    S, m = bin_scene()
    ii = inlet(m, massRate=1.0)
    # RandomInlet::critDt: generator.critDt(density, young) = spherePWaveDt(dRange[0], ...)
    assert ii.critDt() == pytest.approx(0.008 / math.sqrt(1e7 / 2500))
    S.engines = S.engines + [ii]
    S._prepare_dt()
    assert S.dt == pytest.approx(0.9 * 0.006 / math.sqrt(1e7 / 2500)) or S.dt <= 0.9 * ii.critDt()
    with pytest.raises(RuntimeError, match="doneHook"):
        S2, m2 = bin_scene(engines=[inlet(m, massRate=1.0, doneHook="print(1)")])
        S2._engine()


def test_energy_random_inlet_then_outlet(monkeypatch):
    """py/tests/test_energy.py:50-67: an inlet shoots one sphere into an empty field and an outlet
    deletes it in the same step; kinInlet = -Ek, kinOutlet = Ek, and the energies sum to zero.  (The
    reference's engine list is [InsertionSortCollider, BoxInlet, BoxOutlet]; here the GPU engine's trio
    stands in for the collider.)"""
    from woo_gb300 import utils
    mat = utils.defaultMaterial()
    vel, rad = 1., .1
    m = mat.density * (4 / 3.) * math.pi * rad ** 3
    Ek = .5 * m * vel ** 2
    S = Scene(fields=[dem.DemField(gravity=(0, 0, 0))], trackEnergy=True)
    S.engines = dem.DemField.minimalEngines(dynDtPeriod=0) + [
        dem.BoxInlet(maxNum=1, materials=[mat], generator=dem.MinMaxSphereGenerator(dRange=(2 * rad, 2 * rad)),
                     shooter=dem.AlignedMinMaxShooter(dir=(1, 0, 0), vRange=(vel, vel)),
                     box=((-.5, -.5, -.5), (.5, .5, .5)), massRate=0),
        dem.BoxOutlet(inside=True, box=((-1, -1, -1), (1, 1, 1))),
    ]
    S.dt = .05
    run_on_oracle(monkeypatch, S, 1)
    assert len(S.dem.par) == 0
    assert S.energy["kinOutlet"] == Ek
    assert S.energy["kinInlet"] == -Ek
    assert S.energy.total() == 0.


def test_sphere_pack_grid_matches_brute_force():
    from woo_gb300.inlet import _SpherePack
    rng = np.random.default_rng(7)
    C = rng.uniform(-0.3, 0.2, (3000, 3))
    R = rng.uniform(0.002, 0.01, 3000)
    pk = _SpherePack(C, R, rmax=0.012)
    allC, allR = list(C), list(R)
    hits = 0
    for k in range(3000):
        c = rng.uniform(-0.32, 0.22, 3)
        r = rng.uniform(0.002, 0.012)
        if k % 3 == 0:                                    # near-touching: exactly at the sum of radii
            j = rng.integers(len(allR))
            u = rng.normal(size=3)
            c = allC[j] + u / np.linalg.norm(u) * (allR[j] + r)
        A, B = np.array(allC), np.array(allR)
        d = A - c
        brute = bool(np.any(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2] < (B + r) * (B + r)))
        assert pk.overlaps(c, r) == brute
        hits += brute
        if not brute and k % 2:
            pk.add(c, r)
            allC.append(c)
            allR.append(r)
    assert 100 < hits < 2900


def test_generator_psd(monkeypatch):
    S, m = bin_scene(gravity=(0, 0, 0))
    ii = inlet(m, massRate=0, maxAttempts=300, seed=2, box=((-0.02, -0.02, 0.1), (0.02, 0.02, 0.14)))
    S.engines = S.engines + [ii]
    run_on_oracle(monkeypatch, S, 1)
    d, f = ii.generator.psd(num=10)
    assert len(d) == 10 and f[-1] == pytest.approx(1.0) and all(a <= b for a, b in zip(f, f[1:]))
    dm = ii.generator.diamMass()
    assert min(d) == pytest.approx(min(dm[0])) and max(d) == pytest.approx(max(dm[0]))
    _, cnt = ii.generator.psd(mass=False, normalize=False, cumulative=True, num=10)
    assert cnt[-1] == ii.num


def test_angle_inside_cases():
    from woo_gb300.outlet import angle_inside
    assert angle_inside(0.1, 0., 1.) and not angle_inside(-0.1, 0., 1.)
    assert angle_inside(0., 1.5 * math.pi, 0.5 * math.pi)      # interval across 0 (a > b)
    assert not angle_inside(math.pi, 1.5 * math.pi, 0.5 * math.pi)
    assert angle_inside(123., 0., 2 * math.pi)                   # the whole circle
    assert angle_inside(0.3 + 2 * math.pi, 0., 1.)               # phi wraps


def _node(pos, angle):
    return dem.Node(pos=pos, ori=(math.cos(angle / 2), 0, 0, math.sin(angle / 2)))


def test_cylinder_and_arc_inlets_place_inside(monkeypatch):
    from woo_gb300.outlet import cart2cyl, glob2loc
    m = dem.FrictMat(density=2500, young=1e7)
    gen = lambda: dem.MinMaxSphereGenerator(dRange=(0.006, 0.01))
    cyl = dem.CylinderInlet(node=_node((0.3, 0.1, 0.5), 0.7), height=0.1, radius=0.04, massRate=0, maxAttempts=200,
                            materials=[m], generator=gen(), seed=1)
    arc = dem.ArcInlet(node=_node((-0.3, 0.0, 0.5), 0.2), cylBox=((0.05, 0.3, 0.0), (0.12, 1.8, 0.05)), massRate=0,
                       maxAttempts=200, materials=[m], generator=gen(), seed=2)
    box2 = dem.BoxInlet2d(box=((-0.05, -0.05, 0.8), (0.05, 0.05, 0.805)), axis=2, massRate=0, maxAttempts=200,
                          materials=[m], generator=gen(), seed=3)
    S, _ = bin_scene(gravity=(0, 0, 0))
    S.engines = S.engines + [cyl, arc, box2]
    run_on_oracle(monkeypatch, S, 1)
    assert cyl.num > 5 and arc.num > 5 and box2.num > 3
    ids = {k: list(v._inserted) for k, v in (("cyl", cyl), ("arc", arc), ("box2", box2))}
    for i in ids["cyl"]:
        p, r = S.dem.par[i].pos, S.dem.par[i].shape.radius
        for c in _box_corners(p, r):
            q = glob2loc(cyl.node, c)
            assert 0 <= q[0] <= 0.1 and q[1] ** 2 + q[2] ** 2 <= 0.04 ** 2
    for i in ids["arc"]:
        p, r = S.dem.par[i].pos, S.dem.par[i].shape.radius
        for c in _box_corners(p, r):
            q = cart2cyl(glob2loc(arc.node, c))
            assert 0.05 <= q[0] <= 0.12 and 0.3 <= q[1] <= 1.8 and 0 <= q[2] <= 0.05
    sticks_out = False
    for i in ids["box2"]:
        p, r = S.dem.par[i].pos, S.dem.par[i].shape.radius
        assert -0.05 <= p[0] - r and p[0] + r <= 0.05 and -0.05 <= p[1] - r and p[1] + r <= 0.05
        sticks_out |= p[2] + r > 0.805 or p[2] - r < 0.8
    assert sticks_out                                             # along the axis the box is not enforced
    allnew = ids["cyl"] + ids["arc"] + ids["box2"]
    assert _no_overlap(S, allnew)


def _box_corners(p, r):
    return [p + r * np.array([sx, sy, sz]) for sx in (-1, 1) for sy in (-1, 1) for sz in (-1, 1)]


def test_arc_outlet(monkeypatch):
    from woo_gb300.outlet import cart2cyl, glob2loc
    node = _node((0.0, 0.0, 0.0), 0.0)
    out = dem.ArcOutlet(node=node, cylBox=((0.0, -0.6, -1.0), (0.04, 0.6, 0.07)), inside=True, stepPeriod=1000)
    S, m = bin_scene(n_pre=25, gravity=(0, 0, 0))
    S.engines = S.engines + [out]
    before = {p.id: p.pos for p in S.dem.par if isinstance(p.shape, dem.Sphere)}
    run_on_oracle(monkeypatch, S, 1)
    gone = {i for i in before if not S.dem.par.exists(i)}
    expect = set()
    for i, p in before.items():
        q = cart2cyl(glob2loc(node, p))
        if q[0] <= 0.04 and -0.6 <= q[1] <= 0.6 and -1 <= q[2] <= 0.07:
            expect.add(i)
    assert gone == expect and 0 < len(gone) < 25
    with pytest.raises(RuntimeError, match="node"):
        dem.ArcOutlet(cylBox=((0, 0, 0), (1, 1, 1)))


def test_psd_generator_follows_the_curve():
    """Discrete number PSD: the bin choice is deterministic and keeps every bin within one particle of
    its share (Psd.cpp:58-114); sanitizePsd drops leading zeros and normalizes."""
    g = dem.PsdSphereGenerator(psdPts=[(0.005, 0), (0.006, 0), (0.01, 20), (0.02, 100)], discrete=True, mass=False)
    assert g.psdPts == [[0.006, 0.], [0.01, .2], [0.02, 1.]]
    m = dem.FrictMat(density=2000)
    rng = np.random.default_rng(0)
    ds = [g(m, 0., rng)[0] for _ in range(200)]
    assert ds[0] == pytest.approx(0.01)                  # the first bin with a positive passing value
    assert set(np.round(ds, 6)) <= {0.01, 0.02}
    n_small = sum(1 for d in ds if d < 0.015)
    assert abs(n_small - 0.2 * 200) <= 1
    # continuous mass PSD: diameters within the curve, mass shares close to it
    g2 = dem.PsdSphereGenerator(psdPts=[(0.004, 0), (0.008, .5), (0.012, 1.)], mass=True)
    ds = [g2(m, 0., rng)[0] for _ in range(400)]
    assert min(ds) >= 0.004 - 1e-12 and max(ds) <= 0.012 + 1e-12
    masses = np.array([d ** 3 for d in ds])
    assert abs(masses[np.array(ds) <= 0.008].sum() / masses.sum() - 0.5) < 0.05
    g2.revokeLast()
    assert len(g2.genDiamMassTime) == 399
    with pytest.raises(RuntimeError, match="increasing"):
        dem.PsdSphereGenerator(psdPts=[(0.01, .5), (0.005, 1.)])


def test_inlet_with_psd_generator(monkeypatch):
    S, m = bin_scene(gravity=(0, 0, 0))
    ii = dem.BoxInlet(box=((-0.05, -0.05, 0.1), (0.05, 0.05, 0.2)), stepPeriod=100, massRate=0, maxAttempts=500,
                      materials=[m], generator=dem.PsdSphereGenerator(psdPts=[(0.006, 0), (0.012, 1.)]), seed=5)
    S.engines = S.engines + [ii]
    run_on_oracle(monkeypatch, S, 1)
    assert ii.num > 20
    new = list(range(5, len(S.dem.par)))
    assert _no_overlap(S, new)
    r = np.array([S.dem.par[i].shape.radius for i in new])
    assert r.min() >= 0.003 - 1e-12 and r.max() <= 0.006 + 1e-12


def test_placed_particles_stay_when_attempts_run_out(monkeypatch):
    """atMaxAttempts='error' raises, but what was placed before in that run stays (Inlet.cpp:313, 495)."""
    S, m = bin_scene(gravity=(0, 0, 0))
    ii = inlet(m, massRate=50.0, maxAttempts=40, seed=2, box=((-0.02, -0.02, 0.1), (0.02, 0.02, 0.13)))
    S.engines = S.engines + [ii]
    n0 = len(S.dem.par)
    with pytest.raises(RuntimeError, match="maxAttempts reached"):
        run_on_oracle(monkeypatch, S, 101)
    assert ii.num > 0 and len(S.dem.par) == n0 + ii.num


def test_scene_save_load_continues(monkeypatch, tmp_path):
    """Scene.save / Scene.load mid-run (with an inlet and an outlet): the loaded scene continues exactly
    like the original (particles, real contacts with history, host-engine counters, energies)."""
    def make():
        S, m = bin_scene(n_pre=20, trackEnergy=True)
        ii = inlet(m, massRate=1.0, maxNum=25, seed=9, shooter=dem.AlignedMinMaxShooter(dir=(0, 0, -1), vRange=(0.1, 0.3)))
        out = dem.BoxOutlet(box=((0.03, -1, -1), (1, 1, 1)), inside=True, stepPeriod=70)
        S.engines = S.engines + [ii, out]
        return S
    A = make()
    run_on_oracle(monkeypatch, A, 801)
    path = tmp_path / "scene.pkl"
    A.save(str(path))
    B = Scene.load(str(path))
    assert B.step == A.step and B.time == A.time and B._gpu._h is None
    run_on_oracle(monkeypatch, A, 700)
    run_on_oracle(monkeypatch, B, 700)
    assert A.step == B.step == 1501 and A.time == B.time
    ia, oa = A.engines[-2], A.engines[-1]
    ib, ob = B.engines[-2], B.engines[-1]
    assert (ia.num, ia.mass, oa.num, oa.mass) == (ib.num, ib.mass, ob.num, ob.mass)
    assert ia.num > 0 and oa.num > 0
    assert [p.id for p in A.dem.par] == [p.id for p in B.dem.par]
    for p in A.dem.par:
        q = B.dem.par[p.id]
        assert np.array_equal(p.pos, q.pos) and np.array_equal(p.vel, q.vel) and np.array_equal(p.angVel, q.angVel)
    ca, cb = A.dem._contacts(), B.dem._contacts()
    ra, rb = ca.real.astype(bool), cb.real.astype(bool)
    assert ra.sum() > 5 and np.array_equal(ca.keys()[ra], cb.keys()[rb])
    for name in ("force", "trsf", "contPt", "kn", "kt"):
        assert np.array_equal(getattr(ca, name)[ra], getattr(cb, name)[rb]), name
    ea, eb = A.energy, B.energy
    for k in ("grav", "nonviscDamp", "kinInlet"):
        assert eb[k] == pytest.approx(ea[k], rel=1e-12), k
