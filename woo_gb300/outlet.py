"""Outlets (woo.dem.Outlet, src/dem/Outlet.hpp / Outlet.cpp): periodic engines that delete (or mark)
the particles found outside (or inside) a volume, with the bookkeeping of the deleted mass.

They run on the host between GPU steps.  The scene stops the GPU after the contact pass of each step at
which an outlet is due (PeriodicEngine::isActivated, src/core/Engine.cpp:170-195) and runs the outlet
with Scene.step, Scene.time, Scene.dt and Cell.gradV as the engines of that step see them in Woo.
Deleting a particle removes its contacts and leaves its id empty; the other particles keep their ids
and their contact history (DemField::removeParticle, src/dem/Particle.cpp:483-530).

Uninodal particles only (no clumps).  BoxOutlet, StackedBoxOutlet, ArcOutlet and CrazyOutlet are
provided.
"""
import math

import numpy as np

from . import dem

nan = float("nan")


def _fdiv(a, b):
    """a / b in IEEE arithmetic (inf or NaN for b == 0), as the C++ division gives."""
    with np.errstate(divide="ignore", invalid="ignore"):
        return float(np.float64(a) / np.float64(b))


def rotation_matrix(q):
    """Rotation matrix of the unit quaternion (w, x, y, z), Eigen's Quaternion::toRotationMatrix."""
    w, x, y, z = (float(v) for v in q)
    tx, ty, tz = 2 * x, 2 * y, 2 * z
    twx, twy, twz = tx * w, ty * w, tz * w
    txx, txy, txz = tx * x, ty * x, tz * x
    tyy, tyz, tzz = ty * y, tz * y, tz * z
    return np.array([[1 - (tyy + tzz), txy - twz, txz + twy],
                     [txy + twz, 1 - (txx + tzz), tyz - twx],
                     [txz - twy, tyz + twx, 1 - (txx + tyy)]])


def _rotate(q, v):
    return rotation_matrix(q) @ np.asarray(v, np.float64)


def glob2loc(node, p):
    """Node::glob2loc: ori^-1 * (p - pos)."""
    q = np.asarray(node.ori, np.float64)
    qc = np.array([q[0], -q[1], -q[2], -q[3]])
    return _rotate(qc, np.asarray(p, np.float64) - node.pos)


def matvec_rows(M, P):
    """M @ p for every row p of P (n x 3), each component summed left to right."""
    return np.stack([M[i, 0] * P[:, 0] + M[i, 1] * P[:, 1] + M[i, 2] * P[:, 2] for i in range(3)], axis=1)


def sqnorm_rows(V):
    return V[:, 0] * V[:, 0] + V[:, 1] * V[:, 1] + V[:, 2] * V[:, 2]


def glob2loc_rows(node, P):
    q = np.asarray(node.ori, np.float64)
    return matvec_rows(rotation_matrix([q[0], -q[1], -q[2], -q[3]]), P - np.asarray(node.pos, np.float64))


class CellView:
    """What the outlets need of Cell (src/core/Cell.hpp:72-103, Cell.cpp:36-58, 81-120), homoDeform gradV2:
    canonicalizePt and the fluctuation velocities."""

    def __init__(self, hSize, gradV):
        self.hSize = np.asarray(hSize, np.float64).reshape(3, 3)
        self.gradV = np.asarray(gradV, np.float64).reshape(3, 3)
        self.size = np.array([math.sqrt(float(self.hSize[:, i] @ self.hSize[:, i])) for i in range(3)])
        self.shearTrsf = self.hSize / self.size[None, :]
        self.unshearTrsf = np.linalg.inv(self.shearTrsf)
        W = .5 * (self.gradV - self.gradV.T)
        # leviCivita (src/supp/base/Math.hpp:223-228): (m12-m21, m20-m02, m01-m10)
        self.spinVec = .5 * np.array([W[1, 2] - W[2, 1], W[2, 0] - W[0, 2], W[0, 1] - W[1, 0]])

    def canonicalizePt(self, p):
        """shearPt(wrapPt(unshearPt(p))), wrapNum(x, sz) = (x/sz - floor(x/sz))*sz (CompUtils.hpp:10)."""
        return self.canonicalize_rows(np.asarray(p, np.float64).reshape(1, 3))[0]

    def canonicalize_rows(self, P):
        U = matvec_rows(self.unshearTrsf, P)
        nrm = U / self.size[None, :]
        return matvec_rows(self.shearTrsf, (nrm - np.floor(nrm)) * self.size[None, :])

    def pprevFluctVel(self, pos, vel, dt):
        """Cell::pprevFluctVel, HOMO_GRADV2: vel - gradV*(pos - dt/2*vel)."""
        return vel - self.gradV @ (pos - dt / 2 * vel)

    def pprevFluctAngVel(self, angVel):
        return angVel - self.spinVec


def kinetic_energy(mass, inertia, pos, vel, angVel, ori, dt, cell=None):
    """DemData::getEk_any with trans and rot (src/dem/Particle.cpp:247-265)."""
    fv = cell.pprevFluctVel(pos, vel, dt) if cell is not None else np.asarray(vel, np.float64)
    etrans = .5 * (mass * float(fv @ fv))
    T = rotation_matrix(ori)
    fa = cell.pprevFluctAngVel(angVel) if cell is not None else np.asarray(angVel, np.float64)
    erot = .5 * float(fa @ ((T.T @ np.diag(inertia) @ T) @ fa))
    return etrans + erot


def psd(items, cumulative, normalize, num, dRange, diameter, weight, emptyOk=False):
    """DemFuncs::psd (src/dem/Funcs.hpp:61-102): `num` points (diameter, weight in the bins up to it).
    Without a valid dRange it spans the diameters given.  Items with a NaN diameter or weight, or zero
    weight, are left out; items above the range count in the total weight only.  An item goes to bin
    1 + int((num-1)*(d-d0)/(d1-d0)), clamped to [0, num-1]."""
    d0, d1 = (float(x) for x in dRange)
    if math.isnan(d0) or math.isnan(d1) or d0 < 0 or d1 <= 0 or d0 >= d1:
        d0, d1 = math.inf, -math.inf
        for n, it in enumerate(items):
            d = diameter(it, n)
            if d < d0:
                d0 = d
            if d > d1:
                d1 = d
        if math.isinf(d0):
            if not emptyOk:
                raise RuntimeError("DemFuncs::psd: no spherical particles?")
            return [[0., 0.], [0., 0.]]
    ret = [[0., 0.] for _ in range(num)]
    total = 0.
    for n, it in enumerate(items):
        d, w = diameter(it, n), weight(it, n)
        if math.isnan(d) or math.isnan(w) or w == 0.:
            continue
        total += w
        if d > d1:
            continue
        x = (num - 1) * _fdiv(d - d0, d1 - d0)
        # all diameters equal: 0/0; the reference casts the NaN to int, which x86 turns into INT_MIN,
        # so the item lands in bin 0
        b = 0 if math.isnan(x) else max(0, min(num - 1, 1 + int(x)))
        ret[b][1] += w
    for i in range(num):
        ret[i][0] = d0 + _fdiv(i * (d1 - d0), num - 1)
    if normalize:
        for i in range(num):
            ret[i][1] = _fdiv(ret[i][1], total)
    if cumulative:
        for i in range(1, num):
            ret[i][1] += ret[i - 1][1]
    return ret


def _seq_to_py(rows, zipped):
    """DemFuncs::seqVectorToPy: a tuple of per-component lists, or a list of rows when zipped."""
    if zipped:
        return [tuple(r) for r in rows]
    return tuple(list(c) for c in zip(*rows)) if rows else ()


def _t_ok(tRange, t):
    t0, t1 = (float(x) for x in tRange)
    return math.isnan(t0) or math.isnan(t1) or (t0 <= t < t1)


class Outlet(dem.PeriodicEngine):
    """Outlet (src/dem/Outlet.hpp:12-48, Outlet::run Outlet.cpp:15-116): every activation deletes the
    particles whose node lies outside the volume (inside it with inside=True), or with markMask != 0
    only adds markMask to their Particle.mask.  mask != 0 limits it to particles sharing a bit with
    mask.  num and mass count the deleted (marked) particles; with save, diamMassTime gets
    (diameter, mass, Scene.time) of each; currRate is the mass rate, smoothed by currRateSmooth."""
    _defaults = dict(markMask=0, mask=dem.DemField.defaultOutletMask, inside=False, save=False,
                     recoverRadius=False, num=0, savePar=False, mass=0.0, glColor=0.0, glHideZero=False,
                     currRate=nan, currRateSmooth=1.0)

    def __init__(self, **kw):
        super().__init__(**kw)
        self.rDivR0 = []
        self.locs = []
        self.par = []
        self._diamMassTime = []

    def isInside(self, node_pos, node_vel):
        """(inside?, loc) of a point; loc is -1 unless the outlet subdivides its volume."""
        raise RuntimeError(f"{type(self).__name__} did not override Outlet::isInside.")

    def inside_rows(self, P, V):
        """isInside for every row of P (positions) and V (velocities): (bool array, loc array)."""
        res = [self.isInside(P[i], V[i]) for i in range(len(P))]
        return np.array([r[0] for r in res], bool), np.array([r[1] for r in res], np.int64)

    def _select(self, field, cell):
        """Particles to delete/mark, by increasing id (the std::set of Outlet.cpp:18), with their loc;
        only particles whose node is in DemField.nodes are looked at (Outlet.cpp:21)."""
        deleting = self.markMask == 0
        arr = field._arrays
        if arr is not None:
            ids = np.nonzero(field._moving)[0]
            P, V, masks = arr.pos[ids], arr.vel[ids], arr.mask[ids].astype(np.int64)
        else:
            par = [p for p in field.par if getattr(p, "_integrated", True)]
            ids = np.array([p.id for p in par], np.int64)
            P = np.array([p.pos for p in par]).reshape(-1, 3)
            V = np.array([p.vel for p in par]).reshape(-1, 3)
            masks = np.array([p.mask for p in par], np.int64)
        if len(ids) == 0:
            return []
        if cell is not None:
            P = cell.canonicalize_rows(P)
        inside, loc = self.inside_rows(P, V)
        sel = inside == bool(self.inside)
        if self.mask:
            sel &= (masks & self.mask) != 0
        if not deleting:
            sel &= (masks & self.markMask) != self.markMask
        return list(zip(ids[sel].tolist(), loc[sel].tolist()))

    def run(self, scene):
        field = scene.dem
        if field._stale:
            field._engine._download_particles(field)
        cell = CellView(scene.cell.hSize, scene.cell.gradV) if getattr(scene, "periodic", False) else None
        deleting = self.markMask == 0
        if self.recoverRadius and not deleting:
            raise RuntimeError("Outlet.recoverRadius with markMask (a radius change of a live particle) is not supported")
        arr = field._arrays
        step_mass = 0.
        gone = []
        for i, loc in self._select(field, cell):
            p = field.par[i]
            m = float(arr.mass[i]) if arr is not None else p.mass
            if deleting and scene.trackEnergy:
                ek = kinetic_energy(m, arr.inertia[i], arr.pos[i], arr.vel[i], arr.angVel[i], arr.ori[i], scene.dt, cell) \
                    if arr is not None else kinetic_energy(m, p.inertia, p.pos, p.vel, p.angVel, p.ori, scene.dt, cell)
                scene._energy_add("kinOutlet", ek)
            self.num += 1
            self.mass += m
            step_mass += m
            if self.recoverRadius and isinstance(p.shape, dem.Sphere):
                r = (3 * m / (4 * math.pi * p.material.density)) ** (1. / 3.)
                self.rDivR0.append(p.shape.radius / r)
                p.shape.radius = r
                if self.save:
                    self._diamMassTime.append((2 * r, m, scene.time))
            elif self.save:
                self._diamMassTime.append((2 * _equiv_radius(p.shape), m, scene.time))
            self.locs.append(loc)
            if self.savePar:
                self.par.append(p)
            if deleting:
                gone.append(i)
            else:
                p.mask = p.mask | self.markMask
        if gone:
            field.par.remove(gone)
        # the rate over the steps since the previous run; the first run divides by zero steps, as in Woo
        steps = self.stepPeriod if (self.stepPrev < 0 and self.stepPeriod > 0) else scene.step - self.stepPrev
        rate = _fdiv(step_mass, steps * scene.dt)
        if math.isnan(rate) and scene.step > 0:
            rate = 0.
        if math.isnan(self.currRate) or self.stepPrev < 0:
            self.currRate = rate
        else:
            self.currRate = (1 - self.currRateSmooth) * self.currRate + self.currRateSmooth * rate

    # --- python API of Outlet (Outlet.hpp:38-43)
    def clear(self):
        self._diamMassTime = []
        self.rDivR0 = []
        self.locs = []
        self.par = []
        self.mass = 0.
        self.num = 0

    def diamMass(self, zipped=False):
        if zipped:
            return [(d, m) for d, m, _ in self._diamMassTime]
        return (np.array([d for d, _, _ in self._diamMassTime]), np.array([m for _, m, _ in self._diamMassTime]))

    def diamMassTime(self, zipped=False):
        if zipped:
            return list(self._diamMassTime)
        a = np.array(self._diamMassTime).reshape(-1, 3)
        return (a[:, 0].copy(), a[:, 1].copy(), a[:, 2].copy())

    def massOfDiam(self, min=0, max=math.inf):
        ret = 0.
        for d, m, _ in self._diamMassTime:
            if d >= min and d <= max:
                ret += m
        return ret

    def psd(self, mass=True, cumulative=True, normalize=True, num=80, dRange=(nan, nan), tRange=(nan, nan),
            zip=False, emptyOk=False, locs=()):
        """Outlet.psd (Outlet.cpp:132-148): size distribution of the deleted particles, by mass or count,
        within the time range tRange and, when locs is given, from those locations only."""
        if not self.save:
            raise RuntimeError("Outlet.psd(): Outlet.save must be True.")
        want = set(int(x) for x in locs)

        def diameter(dmt, i):
            ok = _t_ok(tRange, dmt[2]) and (not want or (i < len(self.locs) and self.locs[i] in want))
            return dmt[0] if ok else nan

        rows = psd(self._diamMassTime, cumulative, normalize, int(num), dRange, diameter,
                   lambda dmt, i: dmt[1] if mass else 1., emptyOk=emptyOk)
        return _seq_to_py(rows, zip)


def _equiv_radius(shape):
    if isinstance(shape, dem.Sphere):
        return shape.radius
    if isinstance(shape, dem.Ellipsoid):
        return shape.equivRadius()
    return nan


def _box_contains(box, p):
    """AlignedBox3r::contains: min <= p <= max on every axis (closed box)."""
    lo, hi = box
    return bool(lo[0] <= p[0] and lo[1] <= p[1] and lo[2] <= p[2] and p[0] <= hi[0] and p[1] <= hi[1] and p[2] <= hi[2])


class BoxOutlet(Outlet):
    """BoxOutlet (Outlet.hpp:52-62): box = (lower corner, upper corner), in the local coordinates of
    node when one is given.  The default box is empty."""
    _defaults = dict(box=((math.inf,) * 3, (-math.inf,) * 3), node=None)

    def _box(self):
        lo, hi = self.box
        return np.asarray(lo, np.float64).reshape(3), np.asarray(hi, np.float64).reshape(3)

    def isInside(self, pos, vel):
        p = glob2loc(self.node, pos) if self.node is not None else pos
        return _box_contains(self._box(), p), -1

    def _contains_rows(self, P):
        lo, hi = self._box()
        L = glob2loc_rows(self.node, P) if self.node is not None else P
        return np.all(lo[None, :] <= L, axis=1) & np.all(L <= hi[None, :], axis=1), L

    def inside_rows(self, P, V):
        inside, _ = self._contains_rows(P)
        return inside, np.full(len(P), -1, np.int64)


class StackedBoxOutlet(BoxOutlet):
    """StackedBoxOutlet (Outlet.hpp:77-90, Outlet.cpp:206-224): a BoxOutlet whose box is cut along axis at
    the increasing coordinates divs; loc is the slab index (from loc0) of a point inside."""
    _defaults = dict(divs=(), divColors=(), axis=0, loc0=0)

    def __init__(self, **kw):
        super().__init__(**kw)
        d = [float(x) for x in self.divs]
        for i, x in enumerate(d):
            if math.isnan(x) or math.isinf(x):
                raise RuntimeError(f"StackedBoxOutlet.divs: NaN and Inf not allowed (divs[{i}]={x}).")
            if i > 0 and not (d[i - 1] < x):
                raise RuntimeError(f"StackedBoxOutlet.divs: must be increasing (divs[{i - 1}]={d[i - 1]}, divs[{i}]={x}).")

    def isInside(self, pos, vel):
        p = glob2loc(self.node, pos) if self.node is not None else pos
        if not _box_contains(self._box(), p):
            return False, -1
        loc = int(np.searchsorted(np.asarray(self.divs, np.float64), p[self.axis], side="right"))
        return True, loc + self.loc0

    def inside_rows(self, P, V):
        inside, L = self._contains_rows(P)
        loc = np.searchsorted(np.asarray(self.divs, np.float64), L[:, self.axis], side="right") + self.loc0
        return inside, np.where(inside, loc, -1).astype(np.int64)


class CrazyOutlet(Outlet):
    """CrazyOutlet (Outlet.hpp:65-73, Outlet.cpp:253-259): a point is 'inside' while its node's speed is at
    most limVelNorm, so the default (inside=False) deletes particles moving faster than that."""
    _defaults = dict(limVelNorm=1000.0)

    def isInside(self, pos, vel):
        v = np.asarray(vel, np.float64).reshape(1, 3)
        return bool(sqnorm_rows(v)[0] <= self.limVelNorm * self.limVelNorm), -1

    def inside_rows(self, P, V):
        return sqnorm_rows(V) <= self.limVelNorm * self.limVelNorm, np.full(len(P), -1, np.int64)


def cart2cyl(p):
    """CompUtils::cart2cyl (src/supp/base/CompUtils.cpp:115-117): (rho, phi, z)."""
    return np.array([math.sqrt(p[0] * p[0] + p[1] * p[1]), math.atan2(p[1], p[0]), p[2]])


def cyl2cart(c):
    """CompUtils::cyl2cart (CompUtils.cpp:120-122)."""
    return np.array([c[0] * math.cos(c[1]), c[0] * math.sin(c[1]), c[2]])


def angle_inside(phi, a, b):
    """CompUtils::angleInside (CompUtils.cpp:124-132): phi within the angle interval (a, b)."""
    if abs(a - b) >= 2 * math.pi:
        return True
    if a > b:
        a -= 2 * math.pi
    if a == b:
        return math.fmod(a, 2 * math.pi) == math.fmod(phi, 2 * math.pi)
    x = (phi - a) / (2 * math.pi)
    pphi = (x - math.floor(x)) * (2 * math.pi)
    return pphi < (b - a)


def cyl_box_contains(box, pt):
    """CompUtils::cylCoordBox_contains_cartesian (CompUtils.cpp:145-156): pt cartesian, box in
    cylindrical coordinates ((rho0, phi0, z0), (rho1, phi1, z1))."""
    (lo, hi), c = box, cart2cyl(pt)
    return bool(lo[0] <= c[0] <= hi[0] and angle_inside(c[1], lo[1], hi[1]) and lo[2] <= c[2] <= hi[2])


class ArcOutlet(Outlet):
    """ArcOutlet (Outlet.hpp:92-106, Outlet.cpp:226-237): the volume is a prismatic arc, a box in the
    cylindrical coordinates (rho, phi, z) of node's local frame."""
    _defaults = dict(node=None, cylBox=((0., 0., 0.), (0., 0., 0.)), glSlices=32)

    def __init__(self, **kw):
        super().__init__(**kw)
        lo, hi = self.cylBox
        if (lo[0] <= hi[0] and lo[1] <= hi[1] and lo[2] <= hi[2]) and (lo[0] < 0 or hi[0] < 0):
            raise RuntimeError(f"ArcOutlet.cylBox: radius bounds (x-component) must be non-negative (not {lo[0]}..{hi[0]}).")
        if self.node is None:
            raise RuntimeError("ArcOutlet.node: must not be None.")

    def isInside(self, pos, vel):
        return cyl_box_contains(self.cylBox, glob2loc(self.node, pos)), -1
