"""Outlets (src/dem/Outlet.cpp) and particle removal through the Python surface, on the CPU: the
PeriodicEngine schedule against a step-by-step isActivated loop, the container semantics of removed
ids, and whole scripts (Scene + GpuDemEngine bookkeeping + outlet) run with the engine's handle on the
oracle."""
import copy
import math

import numpy as np
import pytest

from woo_gb300 import dem
from woo_gb300.core import Scene

from oracle_handle import run_on_oracle

R = 0.01


def funnel(n_side=3, layers=3, floor=False, seed=5, extra=None, engines=()):
    """Spheres of radius 1 cm between four side walls (x, y = +-5 cm), falling with random velocities;
    an optional floor at z = 0; `extra` = positions of more spheres appended after the column."""
    rng = np.random.default_rng(seed)
    m = dem.FrictMat(density=2500, young=1e7, ktDivKn=0.2, tanPhi=0.5)
    par = [dem.Wall.make(-0.05, axis=0, sense=1, mat=m), dem.Wall.make(0.05, axis=0, sense=-1, mat=m),
           dem.Wall.make(-0.05, axis=1, sense=1, mat=m), dem.Wall.make(0.05, axis=1, sense=-1, mat=m)]
    if floor:
        par.append(dem.Wall.make(0, axis=2, sense=1, mat=m))
    for k in range(layers):
        for i in range(n_side):
            for j in range(n_side):
                c = (-0.025 + 0.025 * i, -0.025 + 0.025 * j, 0.02 + 0.025 * k)
                v = (rng.uniform(-0.2, 0.2), rng.uniform(-0.2, 0.2), rng.uniform(-1.0, 0.0))
                par.append(dem.Sphere.make(c, R, mat=m, vel=v))
    for c in (extra or []):
        par.append(dem.Sphere.make(c, R, mat=m))
    return Scene(fields=[dem.DemField(gravity=(0, 0, -9.81), par=par)],
                 engines=dem.DemField.minimalEngines(damping=0.2, dynDtPeriod=0) + list(engines), dtSafety=0.9)


# ------------------------------------------------------------------------------------------ schedule
class _Rec(dem.PeriodicEngine):
    def __init__(self, **kw):
        super().__init__(**kw)
        self.fired = []

    def run(self, scene):
        self.fired.append((scene.step, scene.time))


class _StubGpu:
    """Counts the steps the scene asks the GPU for."""

    def __init__(self, dt):
        self.dt = dt
        self.steps = 0
        self._ran_time = 0.0

    def run(self, scene, k):
        assert k >= 1
        self.steps += k
        self._ran_time = k * self.dt


def _naive(eng, s0, n, dt):
    """Woo: isActivated evaluated in every step (Scene::doOneStep), time advancing by dt."""
    e = copy.deepcopy(eng)
    out = []
    for s in range(s0, s0 + n):
        if e._activate(s, s * dt):
            out.append(s)
    return out, e


@pytest.mark.parametrize("seed", range(40))
def test_schedule_matches_step_by_step_activation(seed):
    rng = np.random.default_rng(seed)
    kw = dict(stepPeriod=int(rng.integers(1, 8)), stepModulo=bool(rng.integers(2)), initRun=bool(rng.integers(2)),
              nDo=int(rng.choice([-1, 0, 1, 2, 3])))
    s0 = int(rng.integers(0, 20))
    chunks = [int(x) for x in rng.integers(1, 15, size=int(rng.integers(1, 4)))]
    dt = 0.5
    eng = _Rec(**kw)
    ref, ref_eng = _naive(eng, s0, sum(chunks), dt)
    S = Scene(fields=[dem.DemField()])
    S.dt, S.step, S.time = dt, s0, s0 * dt
    S._gpu = _StubGpu(dt)
    S._host = [eng]
    for c in chunks:
        S.run(c)
    assert [s for s, _ in eng.fired] == ref
    assert all(t == s * dt for s, t in eng.fired)
    assert S.step == s0 + sum(chunks) and S._gpu.steps == sum(chunks)
    assert (eng.nDone, eng.stepLast, eng.stepPrev) == (ref_eng.nDone, ref_eng.stepLast, ref_eng.stepPrev)


def test_time_based_periods_rejected():
    S = funnel(engines=[dem.BoxOutlet(box=((-1, -1, -1), (1, 1, 1)), virtPeriod=0.1)])
    with pytest.raises(RuntimeError, match="virtPeriod"):
        S._engine()


# ------------------------------------------------------------------------------------------ container
def test_container_removed_ids():
    S = funnel()
    par = S.dem.par
    n = len(par)
    assert par.remove(6) is True and par.remove(6) is False
    assert not par.exists(6) and len(par) == n
    with pytest.raises(IndexError, match="No such particle: #6"):
        par[6]
    assert [p.id for p in par] == [i for i in range(n) if i != 6]
    assert par.remove([n - 1, n - 2, 3]) == [True, True, True]
    assert len(par) == n - 2                                      # trailing empty ids are trimmed
    assert par[-1].id == n - 3
    p = dem.Sphere.make((0, 0, 0.5), R)
    assert par.add(p) == 6                                        # findFreeId: the first freed id
    assert par.add(dem.Sphere.make((0, 0, 0.6), R)) == 3
    with pytest.raises(IndexError, match="already has id"):
        par.add(p)


def test_removed_id_is_a_dead_slot_on_the_device():
    S = funnel()
    S.dem.par.remove(7)
    S._prepare_dt()
    g = S._engine()
    g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    view = g._device_view(S.dem, pa)
    assert view.mask[7] == 0 and view.flags[7] & 63 == 63
    assert not view.vel[7].any() and not view.angVel[7].any()
    assert np.array_equal(view.pos[7], pa.pos[4])          # parked on the first live sphere
    assert (view.mask[[i for i in range(pa.n) if i != 7]] != 0).all()


# ------------------------------------------------------------------------------------------ scripts
def test_box_outlet_deletes_and_books(monkeypatch):
    out = dem.BoxOutlet(box=((-1, -1, -0.05), (1, 1, 10)), stepPeriod=50, save=True, savePar=True)
    S = funnel(engines=[out])
    n0 = len(S.dem.par)
    masses = {p.id: p.mass for p in S.dem.par}
    run_on_oracle(monkeypatch, S, 1201)                   # the last step (1200) runs the outlet
    gone = [i for i in range(n0) if not S.dem.par.exists(i)]
    assert out.num == len(gone) > 5
    # a removed particle keeps the state it had when the outlet took it (outside the box), detached
    assert len(out.par) == out.num
    assert all(p.pos[2] < -0.05 and p.shape.nodes[0]._field is None for p in out.par)
    assert out.nDone == 1201 // 50 + 1
    assert out.mass == pytest.approx(sum(masses[i] for i in gone), rel=1e-14)
    d, m, t = out.diamMassTime()
    assert np.all(d == 2 * R) and m.sum() == pytest.approx(out.mass, rel=1e-14)
    assert np.all(np.diff(t) >= 0) and out.massOfDiam(0.019, 0.021) == pytest.approx(out.mass, rel=1e-14)
    assert out.locs == [-1] * out.num
    # every remaining movable particle is inside the box after the outlet's last run
    for p in S.dem.par:
        if isinstance(p.shape, dem.Sphere):
            assert p.pos[2] >= -0.05
    # no contact of a removed particle is left
    ca = S.dem._contacts()
    assert not np.isin(ca.idA, gone).any() and not np.isin(ca.idB, gone).any()
    assert math.isfinite(out.currRate)


def test_removal_does_not_change_the_motion(monkeypatch):
    """A sphere that never touches the others, removed when it has fallen out of the box (at the run of
    step 2100, with ~70 real contacts in the column), leaves the rest of the scene exactly as in the scene
    without it: the contact history of the other particles is kept across the removal and the collider
    rebuild that follows it."""
    out = dem.BoxOutlet(box=((-5, -5, -1), (5, 5, 10)), stepPeriod=300, initRun=False)
    A = funnel(floor=True, layers=6, extra=[(3.0, 0, -0.70)], engines=[out])
    B = funnel(floor=True, layers=6)
    n = len(B.dem.par)
    run_on_oracle(monkeypatch, A, 301)
    assert out.nDone == 1 and out.stepPrev == 0           # step 0 only started the count (initRun=False)
    run_on_oracle(monkeypatch, A, 1500)
    assert out.nDone == 6 and out.num == 0 and A.dem.par.exists(n)
    assert A.dem.con.countReal() > 20
    run_on_oracle(monkeypatch, A, 600)
    assert out.nDone == 8 and out.num == 1 and not A.dem.par.exists(n)
    assert out.stepLast == 2400 and out.stepPrev == 2100
    run_on_oracle(monkeypatch, A, 300)
    run_on_oracle(monkeypatch, B, 2701)
    assert A.step == B.step == 2701
    ca, cb = A.dem._contacts(), B.dem._contacts()
    ra, rb = ca.real.astype(bool), cb.real.astype(bool)
    assert ra.sum() > 50
    assert np.array_equal(ca.keys()[ra], cb.keys()[rb])
    for name in ("force", "trsf", "contPt", "kn", "kt", "stepCreated"):
        assert np.array_equal(getattr(ca, name)[ra], getattr(cb, name)[rb]), name
    for i in range(n):
        assert np.array_equal(A.dem.par[i].pos, B.dem.par[i].pos)
        assert np.array_equal(A.dem.par[i].vel, B.dem.par[i].vel)
        assert np.array_equal(A.dem.par[i].angVel, B.dem.par[i].angVel)


def test_marking_mode(monkeypatch):
    out = dem.BoxOutlet(box=((-1, -1, -0.05), (1, 1, 10)), stepPeriod=40, markMask=16)
    S = funnel(engines=[out])
    n0 = len(S.dem.par)
    run_on_oracle(monkeypatch, S, 801)
    marked = [p.id for p in S.dem.par if p.mask & 16]
    assert len(S.dem.par) == n0 and all(S.dem.par.exists(i) for i in range(n0))
    assert out.num == len(marked) > 3                     # each particle is marked once
    assert all(S.dem.par[i].mask == (dem.DemField.defaultMovableMask | 16) for i in marked)
    assert all(S.dem.par[i].pos[2] < -0.05 for i in marked)


def test_crazy_and_stacked_outlets(monkeypatch):
    crazy = dem.CrazyOutlet(limVelNorm=50.0, stepPeriod=10)
    stacked = dem.StackedBoxOutlet(box=((-1, -1, -10), (1, 1, -0.05)), divs=(-0.3, -0.1), axis=2, loc0=10,
                                   inside=True, stepPeriod=10, save=True)
    S = funnel(engines=[crazy, stacked])
    S.dem.par[8].vel = (0, 0, -60.0)
    run_on_oracle(monkeypatch, S, 1)
    assert crazy.num == 1 and not S.dem.par.exists(8)
    run_on_oracle(monkeypatch, S, 1300)
    assert stacked.num > 5
    assert set(stacked.locs) <= {10, 11, 12} and 12 in stacked.locs
    with pytest.raises(RuntimeError, match="increasing"):
        dem.StackedBoxOutlet(divs=(0.2, 0.1))


def test_kin_outlet_energy(monkeypatch):
    """Scene.energy['kinOutlet'] sums DemData::getEk_any of the deleted particles at their removal."""

    class Snap(dem.PeriodicEngine):
        def run(self, scene):
            f = scene.dem
            if f._stale:
                f._engine._download_particles(f)
            self.states.append(f._arrays.copy())

    snap = Snap(stepPeriod=50)
    snap.states = []
    out = dem.BoxOutlet(box=((-1, -1, -0.05), (1, 1, 10)), stepPeriod=50)
    S = funnel(engines=[snap, out])
    S.trackEnergy = True
    alive = set(range(len(S.dem.par)))
    run_on_oracle(monkeypatch, S, 1001)
    expect = 0.0
    for st in snap.states:
        for i in sorted(alive):
            if i >= 4 and st.pos[i][2] < -0.05:
                v, w = st.vel[i], st.angVel[i]
                expect += .5 * (st.mass[i] * float(v @ v)) + .5 * float(w @ (st.inertia[i] * w))
                alive.discard(i)
    assert out.num == len(set(range(len(snap.states[0].pos))) - alive)
    assert S.energy["kinOutlet"] == pytest.approx(expect, rel=1e-12)


def test_row_tests_match_point_tests():
    """The vectorized volume tests give what isInside gives point by point (rotated local frame,
    stacked slabs, speed limit), and canonicalize_rows wraps into the sheared cell."""
    from woo_gb300 import outlet as O
    rng = np.random.default_rng(0)
    P = rng.uniform(-1.5, 1.5, (400, 3))
    V = rng.normal(0, 30, (400, 3))
    node = dem.Node(pos=(0.1, -0.2, 0.3), ori=(np.cos(0.3), 0, np.sin(0.3), 0))
    for o in (dem.BoxOutlet(box=((-1, -0.5, -1), (0.5, 1, 0.8))),
              dem.BoxOutlet(box=((-1, -0.5, -1), (0.5, 1, 0.8)), node=node),
              dem.StackedBoxOutlet(box=((-1, -1, -1), (1, 1, 1)), divs=(-0.2, 0.4), axis=1, loc0=3, node=node),
              dem.CrazyOutlet(limVelNorm=40.0)):
        ins, loc = o.inside_rows(P, V)
        for i in range(len(P)):
            assert (bool(ins[i]), int(loc[i])) == o.isInside(P[i], V[i])
        assert 0 < ins.sum() < len(P)
    cell = O.CellView(hSize=[[1.0, 0.3, 0.0], [0.0, 1.2, 0.0], [0.0, 0.0, 0.9]], gradV=np.zeros((3, 3)))
    W = cell.canonicalize_rows(P * 3)
    U = (np.linalg.inv(cell.shearTrsf) @ W.T).T
    assert np.all(U >= -1e-12) and np.all(U <= cell.size[None, :] + 1e-12)
    # the wrapped point is the original one shifted by whole cell vectors
    k = np.linalg.solve(cell.hSize, (P * 3 - W).T).T
    assert np.allclose(k, np.round(k), atol=1e-9)


def test_psd_known_answer():
    """DemFuncs::psd on four diameters: bins 1 + int(3*(d-1)/3) -> 1, 2, 3, 3."""
    from woo_gb300.outlet import psd
    items = [(1., 1., 0.), (2., 1., 0.), (3., 1., 0.), (4., 1., 0.)]
    rows = psd(items, True, True, 4, (math.nan, math.nan), lambda it, i: it[0], lambda it, i: it[1])
    assert rows == [[1., 0.], [2., .25], [3., .5], [4., 1.]]
    rows = psd(items, False, False, 4, (math.nan, math.nan), lambda it, i: it[0], lambda it, i: it[1])
    assert [r[1] for r in rows] == [0., 1., 1., 2.]
    # above the given range: counted in the total only
    rows = psd(items, False, True, 3, (1., 3.), lambda it, i: it[0], lambda it, i: it[1])
    assert [r[1] for r in rows] == [0., .25, .5]
    with pytest.raises(RuntimeError, match="no spherical"):
        psd([], True, True, 4, (math.nan, math.nan), lambda it, i: it[0], lambda it, i: it[1])
    assert psd([], True, True, 4, (math.nan, math.nan), None, None, emptyOk=True) == [[0., 0.], [0., 0.]]


def test_outlet_psd_filters(monkeypatch):
    out = dem.StackedBoxOutlet(box=((-1, -1, -10), (1, 1, -0.05)), divs=(-0.3,), axis=2, inside=True,
                               stepPeriod=10, save=True)
    S = funnel(engines=[out])
    run_on_oracle(monkeypatch, S, 1300)
    d, f = out.psd()
    assert len(d) == 80 and f[-1] == pytest.approx(1.0)
    kw = dict(cumulative=False, normalize=False, dRange=(0.015, 0.025), num=5)
    by_loc = [out.psd(locs=[k], **kw)[1] for k in (0, 1)]
    total = out.psd(**kw)[1]
    assert np.allclose(np.add(by_loc[0], by_loc[1]), total)
    assert sum(total) == pytest.approx(out.mass) and set(out.locs) <= {0, 1}
    assert out.psd(locs=[0], emptyOk=True, **kw)[1] == by_loc[0]
    with pytest.raises(RuntimeError, match="save"):
        dem.BoxOutlet().psd()


def test_periodic_outlet_canonical_positions_and_fluctuation_energy(monkeypatch):
    """A sheared periodic cell: the outlet tests canonicalized positions (Outlet.cpp:20-24) and books
    kinOutlet from the fluctuation velocities with the step's own gradV (Particle.cpp:247-265)."""
    from woo_gb300 import utils

    class Snap(dem.PeriodicEngine):
        def run(self, scene):
            f = scene.dem
            if f._stale:
                f._engine._download_particles(f)
            self.states.append((scene.step, f._arrays.copy(), scene.cell.hSize, scene.cell.gradV, scene.dt,
                                [p.id for p in f.par]))

    rng = np.random.default_rng(5)
    m = dem.FrictMat(density=1e3, young=1e6, ktDivKn=.2, tanPhi=.4)
    snap = Snap(stepPeriod=25)
    snap.states = []
    out = dem.BoxOutlet(box=((-10, -10, 0.0), (10, 10, 1.2)), inside=True, stepPeriod=25)
    S = Scene(fields=[dem.DemField(gravity=(0, 0, 0))],
              engines=utils.defaultEngines(damping=.2, dynDtPeriod=0) + [snap, out], dtSafety=.5, trackEnergy=True)
    S.periodic = True
    S.cell.setBox(4, 4, 4)
    S.cell.nextGradV = np.array([[0, 0, 0.2], [0, 0, 0], [0, 0, 0]])
    for ix in range(4):
        for iy in range(4):
            for iz in range(4):
                c = np.array([ix, iy, iz]) + .5 + rng.uniform(-.05, .05, 3)
                S.dem.par.add(utils.sphere(c, .45, mat=m, vel=rng.normal(0, .3, 3)))
    run_on_oracle(monkeypatch, S, 101)
    assert out.nDone == 5 and out.num > 10
    expect_gone, expect_ek = [], 0.0
    alive = set(range(64))
    for step, st, hsize, gradv, dt, live in snap.states:
        for i in sorted(set(live) & alive):
            frac = np.linalg.solve(hsize, st.pos[i])
            z = (hsize @ (frac - np.floor(frac)))[2]
            if 0.0 <= z <= 1.2:
                expect_gone.append(i)
                alive.discard(i)
                v = st.vel[i] - gradv @ (st.pos[i] - dt / 2 * st.vel[i])
                W = .5 * (gradv - gradv.T)
                spin = .5 * np.array([W[1, 2] - W[2, 1], W[2, 0] - W[0, 2], W[0, 1] - W[1, 0]])
                w = st.angVel[i] - spin
                expect_ek += .5 * st.mass[i] * float(v @ v) + .5 * float(w @ (st.inertia[i] * w))
    assert sorted(expect_gone) == sorted(i for i in range(64) if not S.dem.par.exists(i))
    assert S.energy["kinOutlet"] == pytest.approx(expect_ek, rel=1e-10)
    assert any(np.any(g != 0) for _, _, _, g, _, _ in snap.states)   # the shear was on while the outlet ran


def test_dead_slots_spread_over_live_spheres():
    S = funnel()
    S.dem.par.remove(list(range(4, 20)))
    S._prepare_dt()
    g = S._engine()
    g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    view = g._device_view(S.dem, pa)
    parked = {tuple(view.pos[i]) for i in range(4, 20)}
    live = {tuple(pa.pos[i]) for i in range(20, 31)}
    assert parked <= live and len(parked) == 11              # 16 dead slots over the 11 live spheres


def test_disappear_and_reappear(monkeypatch):
    """ParticleContainer.disappear / reappear (ParticleContainer.cpp:239-273): a resting sphere loses its
    contacts with the new mask and falls through the floor; reappearing restores its mask."""
    S = funnel(floor=True, layers=1, n_side=1)
    run_on_oracle(monkeypatch, S, 3000)
    sid = 5
    assert S.dem.con.existsReal(4, sid)                   # resting on the floor
    S.dem.par.disappear([sid], mask=0b1000)
    assert not S.dem.con.exists(4, sid)
    assert S.dem.par[sid].mask == 0b1000 and S.dem.par[sid].shape.visible is False
    run_on_oracle(monkeypatch, S, 400)
    assert S.dem.par[sid].pos[2] < 0                      # no contact with the floor any more
    S.dem.par.reappear([sid], mask=dem.DemField.defaultMovableMask)
    assert S.dem.par[sid].mask == dem.DemField.defaultMovableMask and S.dem.par[sid].shape.visible is True
    with pytest.raises(RuntimeError, match="removeOverlapping"):
        S.dem.par.reappear([sid], mask=5, removeOverlapping=True)
    with pytest.raises(IndexError):
        S.dem.par.disappear([999], mask=0)


def test_contact_container_clear(monkeypatch):
    S = funnel(floor=True, layers=2)
    run_on_oracle(monkeypatch, S, 2500)
    assert S.dem.con.countReal() > 3
    S.dem.con.clear()
    assert len(S.dem.con) == 0
    run_on_oracle(monkeypatch, S, 1)
    assert S.dem.con.countReal() > 3                      # found again, with fresh history
    assert all(c.stepCreated == 2500 for c in S.dem.con)
