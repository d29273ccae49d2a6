"""Inlets (woo.dem.Inlet, src/dem/Inlet.hpp / Inlet.cpp): periodic engines that insert new spheres
into a running scene at a prescribed mass rate.

They run on the host between GPU steps, scheduled like the outlets (PeriodicEngine::isActivated,
src/core/Engine.cpp:170-195).  New particles take the ids that removed particles left (findFreeId)
or are appended; the GPU engine uploads them, with the contact history of the others, before its
next step.  The sphere generator, the placement test and the mass bookkeeping follow
RandomInlet::run (Inlet.cpp:228-515) for a spheres-only generator:

- the goal mass grows by massRate*dt*(steps since the previous run); particles are made until the
  generated mass reaches it (or, for massRate <= 0, until maxAttempts placements fail);
- a particle is placed at random positions inside the box shrunk by padDist until it overlaps none of
  the spheres near the box (existing ones and the ones placed in this run), trying a new particle
  every maxAttempts/attemptPar attempts; atMaxAttempts decides what a failure does;
- maxMass / maxNum end the inlet (dead, currRate zeroed when zeroRateAtStop).

Inlet volumes: BoxInlet, BoxInlet2d, CylinderInlet, ArcInlet.  Random numbers come from a numpy
generator seeded by `seed` (Woo draws from the C library's rand(), so its placements cannot be
reproduced anyway).  Generators: MinMaxSphereGenerator, PsdSphereGenerator.  Not provided: clump
generators, spatial biases, periodic cells, doneHook strings.
"""
import math

import numpy as np

from . import dem

nan = float("nan")

MAXATT = {"error": 0, "dead": 1, "warn": 2, "silent": 3, "nothing": 3, "ignore": 3, "": 3, "doneHook": 4, "done": 4}


class ParticleGenerator(dem._Attrs):
    """ParticleGenerator (Inlet.hpp:53-86): genDiamMassTime of the generated particles (with save)."""
    _defaults = dict(save=True)

    def __init__(self, **kw):
        super().__init__(**kw)
        self.genDiamMassTime = []

    def revokeLast(self):
        if self.save and self.genDiamMassTime:
            self.genDiamMassTime.pop()

    def clear(self):
        self.genDiamMassTime = []

    def diamMass(self, zipped=False):
        if zipped:
            return [(d, m) for d, m, _ in self.genDiamMassTime]
        return (np.array([d for d, _, _ in self.genDiamMassTime]), np.array([m for _, m, _ in self.genDiamMassTime]))

    def massOfDiam(self, min=0, max=math.inf):
        ret = 0.
        for d, m, _ in self.genDiamMassTime:
            if d >= min and d <= max:
                ret += m
        return ret

    def psd(self, mass=True, cumulative=True, normalize=True, dRange=(nan, nan), tRange=(nan, nan), num=80):
        """ParticleGenerator.psd (Inlet.cpp:165-173): size distribution of the generated particles."""
        from .outlet import psd, _seq_to_py, _t_ok
        if not self.save:
            raise RuntimeError("ParticleGenerator.save must be True for calling ParticleGenerator.psd()")
        rows = psd(self.genDiamMassTime, cumulative, normalize, int(num), dRange,
                   lambda dmt, i: dmt[0] if _t_ok(tRange, dmt[2]) else nan, lambda dmt, i: dmt[1] if mass else 1.)
        return _seq_to_py(rows, False)


class MinMaxSphereGenerator(ParticleGenerator):
    """MinMaxSphereGenerator (Inlet.hpp:88-99, Inlet.cpp:189-200): spheres with diameter uniform in dRange."""
    _defaults = dict(dRange=(nan, nan))

    def isSpheresOnly(self):
        return True

    def padDist(self):
        return min(self.dRange) / 2.

    def minMaxDiam(self):
        return tuple(self.dRange)

    def critDt(self, density, young):
        # DemFuncs::spherePWaveDt(dRange[0], density, young): the reference passes the smaller diameter
        return self.dRange[0] / math.sqrt(young / density)

    def __call__(self, mat, time, rng):
        d0, d1 = (float(x) for x in self.dRange)
        if math.isnan(d0) or math.isnan(d1) or d0 > d1:
            raise RuntimeError("MinMaxSphereGenerator: dRange[0]>dRange[1], or they are NaN!")
        r = .5 * (d0 + rng.random() * (d1 - d0))
        p = dem.Sphere.make((0, 0, 0), r, mat=mat)
        if self.save:
            self.genDiamMassTime.append((2 * r, p.mass, time))
        return 2 * r, [(p, (np.array([-r, -r, -r]), np.array([r, r, r])))]


def sanitize_psd(pts, src):
    """PsdSphereGenerator::sanitizePsd (src/dem/Psd.cpp:23-44): checks, leading zero points and trailing
    repeated maxima dropped, passing values normalized to end at 1."""
    pts = [[float(d), float(f)] for d, f in pts]
    if not pts:
        return pts
    for i in range(len(pts) - 1):
        if pts[i][0] < 0 or pts[i][1] < 0:
            raise RuntimeError(src + ": negative values not allowed.")
        if pts[i][0] > pts[i + 1][0]:
            raise RuntimeError(f"{src}: diameters (the x-component) must be increasing ({pts[i][0]}>={pts[i + 1][0]})")
        if pts[i][1] > pts[i + 1][1]:
            raise RuntimeError(f"{src}: passing values (the y-component) must be increasing ({pts[i][1]}>{pts[i + 1][1]})")
    max_pass = pts[-1][1]
    ii = 0
    while ii < len(pts) and not pts[ii][1] > 0:
        ii += 1
    if ii > 1:
        pts = pts[ii - 1:]
    ii = len(pts) - 2
    while ii >= 0 and not pts[ii][1] < max_pass:
        ii -= 1
    if ii < len(pts) - 2:
        pts = pts[:ii + 2]
    if not pts:
        raise RuntimeError(src + ": empty after removing spurious values?")
    if max_pass != 1.0:
        for v in pts:
            v[1] /= max_pass
    return pts


class PsdSphereGenerator(ParticleGenerator):
    """PsdSphereGenerator (src/dem/Psd.hpp:6-36, Psd.cpp:23-175): spheres following the cumulative PSD
    psdPts (diameter, passing fraction), by mass or by number.  Each new sphere goes to the PSD point
    whose bin is furthest below its share; with `discrete` it takes that point's diameter, otherwise a
    diameter between the previous point and it (inverse-square interpolation for mass PSDs, linear for
    number PSDs)."""
    _defaults = dict(discrete=False, psdPts=(), mass=True)

    def __init__(self, **kw):
        super().__init__(**kw)
        self.psdPts = sanitize_psd(self.psdPts, "PsdSphereGenerator.psdPts")
        self.weightPerBin = [0.] * len(self.psdPts)
        self.weightTotal = 0.
        self._last = None

    def isSpheresOnly(self):
        return True

    def padDist(self):
        return self.psdPts[0][0] / 2. if self.psdPts else nan

    def minMaxDiam(self):
        return (self.psdPts[0][0], self.psdPts[-1][0]) if self.psdPts else (nan, nan)

    def critDt(self, density, young):
        if not self.psdPts:
            return math.inf
        return self.minMaxDiam()[0] / math.sqrt(young / density)

    def clear(self):
        super().clear()
        self.weightTotal = 0.
        self.weightPerBin = [0.] * len(self.psdPts)

    def computeNextRadiusBin(self, rng):
        """PsdSphereGenerator::computeNextRadiusBin (Psd.cpp:58-114)."""
        pts = self.psdPts
        if not pts:
            raise RuntimeError("PsdSphereGenerator.psdPts is empty.")
        max_diff, max_bin = -math.inf, -1
        if self.weightTotal <= 0:
            max_bin = 0
            for i in range(len(pts) - 1):
                if pts[i + 1][1] - pts[i][1] > 0 and pts[i][1] > 0:
                    max_bin = i
                    break
        else:
            for i in range(len(pts)):
                desired = pts[i][1] - (pts[i - 1][1] if i > 0 else 0.)
                diff = desired - self.weightPerBin[i] * 1. / self.weightTotal
                if diff > max_diff and not (self.discrete and desired == 0.):
                    max_diff, max_bin = diff, i
        if self.discrete:
            r = pts[max_bin][0] / 2.
        elif max_bin == 0:
            r = pts[0][0] / 2.
        else:
            a, b = pts[max_bin - 1][0] / 2., pts[max_bin][0] / 2.
            u = rng.random()
            r = math.sqrt(1 / (1 / (a * a) + u * (1 / (b * b) - 1 / (a * a)))) if self.mass else a + u * (b - a)
        return r, max_bin

    def revokeLast(self):
        if self._last is not None:
            b, w = self._last
            self.weightPerBin[b] -= w
            self.weightTotal -= w
        super().revokeLast()

    def __call__(self, mat, time, rng):
        if self.mass and not mat.density > 0:
            raise ValueError(f"PsdSphereGenerator: material density must be positive (not {mat.density})")
        r, b = self.computeNextRadiusBin(rng)
        p = dem.Sphere.make((0, 0, 0), r, mat=mat)
        w = p.mass if self.mass else 1.
        self.weightPerBin[b] += w
        self.weightTotal += w
        self._last = (b, w)
        if self.save:
            self.genDiamMassTime.append((2 * r, p.mass, time))
        return 2 * r, [(p, (np.array([-r, -r, -r]), np.array([r, r, r])))]


class AlignedMinMaxShooter(dem._Attrs):
    """AlignedMinMaxShooter (Inlet.hpp:109-121): velocity dir * U(vRange), no rotation."""
    _defaults = dict(dir=(1.0, 0.0, 0.0), vRange=(nan, nan))

    def __call__(self, node, rng):
        v0, v1 = (float(x) for x in self.vRange)
        if math.isnan(max(v0, v1)):
            raise RuntimeError("AlignedMinMaxShooter.vRange: must not contain NaN.")
        d = np.asarray(self.dir, np.float64)
        d = d / math.sqrt(float(d @ d))
        node.dem.vel = d * (v0 + rng.random() * (v1 - v0))
        node.dem.angVel = (0, 0, 0)


class Inlet(dem.PeriodicEngine):
    """Inlet (Inlet.hpp:15-51): mask of new particles, maxMass / maxNum limits, mass and num generated,
    currRate smoothed by currRateSmooth."""
    _defaults = dict(mask=dem.DemField.defaultInletMask, maxMass=-1.0, maxNum=-1, doneHook="", mass=0.0, num=0,
                     currRate=nan, zeroRateAtStop=True, currRateSmooth=1.0, glColor=0.0)

    def _check(self):
        super()._check()
        if self.doneHook:
            raise RuntimeError(f"{type(self).__name__}.doneHook (a Python string run by Woo) is not supported")

    def setCurrRate(self, rate):
        if math.isnan(self.currRate) or self.stepPrev < 0:
            self.currRate = rate
        else:
            self.currRate = (1 - self.currRateSmooth) * self.currRate + self.currRateSmooth * rate

    def everythingDone(self):
        """Inlet::everythingDone (Inlet.cpp:215-225)."""
        if (self.maxMass > 0 and self.mass >= self.maxMass) or (self.maxNum > 0 and self.num >= self.maxNum):
            self.dead = True
            if self.zeroRateAtStop:
                self.currRate = 0.
            return True
        return False


class _SpherePack:
    """The spheres a new particle must not overlap: |c - s.c|^2 < (s.r + r)^2 is an overlap
    (Inlet.cpp:363-370).  A uniform grid of cell size 2*rmax (rmax bounds every radius, new ones
    included) limits the test to the 27 cells around c, which hold every sphere that can overlap."""

    def __init__(self, C, R, rmax):
        n = len(R)
        self.h = 2. * max(float(rmax), float(R.max()) if n else 0.)
        if not self.h > 0:
            self.h = 1.
        self.C = np.empty((max(2 * n, 64), 3))
        self.R = np.empty(len(self.C))
        self.n = n
        self.C[:n], self.R[:n] = C, R
        self.cells = {}
        if n:
            K = np.floor(C / self.h).astype(np.int64)
            order = np.lexsort((K[:, 2], K[:, 1], K[:, 0]))
            Ks = K[order]
            starts = np.nonzero(np.any(np.diff(Ks, axis=0) != 0, axis=1))[0] + 1
            bounds = np.concatenate([[0], starts, [n]])
            for a, b in zip(bounds[:-1], bounds[1:]):
                self.cells[tuple(Ks[a].tolist())] = order[a:b].tolist()

    def _key(self, c):
        return tuple(int(math.floor(x / self.h)) for x in c)

    def overlaps(self, c, r):
        kx, ky, kz = self._key(c)
        idx = []
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    idx.extend(self.cells.get((kx + dx, ky + dy, kz + dz), ()))
        if not idx:
            return False
        d = self.C[idx] - c[None, :]
        s = self.R[idx] + r
        return bool(np.any(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2] < s * s))

    def add(self, c, r):
        if self.n == len(self.R):
            self.C = np.concatenate([self.C, np.empty_like(self.C)])
            self.R = np.concatenate([self.R, np.empty_like(self.R)])
        self.C[self.n], self.R[self.n] = c, r
        self.cells.setdefault(self._key(c), []).append(self.n)
        self.n += 1


def _box_contains_box(box, b):
    (lo, hi), (blo, bhi) = box, b
    return bool(np.all(lo <= blo) and np.all(bhi <= hi))


def _sq_exterior_distance(box, p):
    lo, hi = box
    d = np.maximum(lo - p, 0.) + np.maximum(p - hi, 0.)
    return float(d @ d)


class RandomInlet(Inlet):
    """RandomInlet (Inlet.hpp:196-241, RandomInlet::run Inlet.cpp:228-515), spheres-only generators."""
    _defaults = dict(massRate=nan, materials=(), generator=None, shooter=None, spatialBias=None, maxAttempts=5000,
                     attemptPar=5, atMaxAttempts="error", padDist=0.0, color=nan, stepGoalMass=0.0,
                     collideExisting=True, seed=0)

    def __init__(self, **kw):
        super().__init__(**kw)
        self._rng = np.random.default_rng(self.seed)
        self._inserted = []

    def _check(self):
        super()._check()
        if self.spatialBias is not None:
            raise RuntimeError("RandomInlet.spatialBias is not supported")

    def critDt(self):
        """RandomInlet::critDt (Inlet.cpp:203-212)."""
        if self.generator is None:
            return math.inf
        ret = math.inf
        for m in self.materials:
            if isinstance(m, dem.ElastMat):
                ret = min(ret, self.generator.critDt(m.density, m.young))
        return ret

    def minMaxDiam(self):
        return self.generator.minMaxDiam() if self.generator is not None else (nan, nan)

    def clear(self):
        if self.generator is not None:
            self.generator.clear()
        self.num = 0
        self.mass = 0.
        self.stepGoalMass = 0.

    def randomPosition(self, diam, padDist):
        raise RuntimeError("Calling RandomInlet.randomPosition (abstract method); use derived classes.")

    def validateBox(self, b):
        raise RuntimeError("Calling RandomInlet.validateBox (abstract method); use derived classes.")

    def _reserve(self):
        """How many particles this inlet may still add (None: no bound known)."""
        if self.maxNum > 0:
            return max(self.maxNum - self.num, 0)
        if self.maxMass > 0 and self.generator is not None and self.materials:
            dmin = float(self.generator.minMaxDiam()[0])
            rho = min(m.density for m in self.materials)
            mmin = (4 / 3.0) * math.pi * (dmin / 2) ** 3 * rho
            if mmin > 0:
                return int(math.ceil(max(self.maxMass - self.mass, 0) / mmin)) + 1
        return None

    def run(self, scene):
        field = scene.dem
        if getattr(scene, "periodic", False):
            raise RuntimeError("RandomInlet in a periodic cell is not supported")
        if self.generator is None:
            raise RuntimeError("RandomInlet.generator==None!")
        if not self.materials:
            raise RuntimeError("RandomInlet.materials is empty!")
        if math.isnan(self.massRate):
            raise RuntimeError(f"RandomInlet.massRate must be given (is {self.massRate}); if you want to generate as "
                               "many particles as possible, say massRate=0.")
        if self.massRate <= 0 and self.maxAttempts == 0:
            raise RuntimeError("RandomInlet.massFlowRate<=0 (no massFlowRate prescribed), but RandomInlet.maxAttempts==0. "
                               "(unlimited number of attempts); this would cause infinite loop.")
        if not self.generator.isSpheresOnly():
            raise RuntimeError("RandomInlet: only spheres-only generators are supported")
        atMax = MAXATT[self.atMaxAttempts] if isinstance(self.atMaxAttempts, str) else int(self.atMaxAttempts)
        rng = self._rng
        self.padDist = self.generator.padDist()
        if math.isnan(self.padDist) or self.padDist < 0:
            raise RuntimeError(f"generator.padDist(): returned invalid value {self.padDist}")
        if self.stepPrev == -1 and self.stepPeriod > 0:
            self.stepPrev = -self.stepPeriod
        nSteps = scene.step - self.stepPrev
        self.stepGoalMass += self.massRate * scene.dt * nSteps
        step_mass = 0.
        # spheres near the inlet: the existing ones, then those placed in this run (Inlet.cpp:259-284)
        pack = _SpherePack(*self._existing_spheres(field), rmax=float(self.generator.minMaxDiam()[1]) / 2.)
        new = []
        done = False
        while True:
            if self.everythingDone():
                done = True
                break
            if self.massRate > 0 and self.mass >= self.stepGoalMass:
                break
            attempt = -1
            placed = None
            while True:
                attempt += 1
                if attempt >= self.maxAttempts:
                    self.generator.revokeLast()
                    if self.massRate <= 0:
                        break
                    if atMax == 0:
                        # the particles placed before are in the scene already (Woo inserts each at once)
                        if new:
                            field.par.add(new, nodes=1)
                            self._inserted.extend(p.id for p in new)
                        raise RuntimeError(f"RandomInlet.maxAttempts reached ({self.maxAttempts})")
                    if atMax == 1:
                        self.dead = True
                        done = True
                    break
                per = self.maxAttempts // self.attemptPar if self.attemptPar else 0
                if attempt == 0 or (per > 0 and attempt % per == 0):
                    if attempt > 0:
                        self.generator.revokeLast()
                    mi = 0
                    if len(self.materials) > 1:
                        # the reference picks max(size*U, size-1): always the last material
                        mi = max(int(len(self.materials) * rng.random()), len(self.materials) - 1)
                    mat = self.materials[mi]
                    diam, pee = self.generator(mat, scene.time, rng)
                pos = self.randomPosition(diam, self.padDist)
                ok = True
                for par, (elo, ehi) in pee:
                    if not self.validateBox((elo + pos, ehi + pos)):
                        ok = False
                        break
                    if pack.overlaps(pos + par.shape.nodes[0]._local["pos"], par.shape.radius):
                        ok = False
                        break
                if ok:
                    for par, _ in pee:
                        pack.add(pos + par.shape.nodes[0]._local["pos"], par.shape.radius)
                    placed = pee
                    break
            if placed is None:
                break
            self.num += 1
            for par, _ in placed:
                par.mask = self.mask
                node = par.shape.nodes[0]
                node.pos = node._local["pos"] + pos
                if self.shooter is not None:
                    self.shooter(node, rng)
                if scene.trackEnergy:
                    from .outlet import kinetic_energy
                    ek = kinetic_energy(node.dem.mass, node.dem.inertia, node.pos, node.dem.vel, node.dem.angVel,
                                        node.ori, scene.dt)
                    scene._energy_add("kinInlet", -ek)
                self.mass += node.dem.mass
                step_mass += node.dem.mass
                new.append(par)
        if new:
            field.par.add(new, nodes=1)
            self._inserted.extend(p.id for p in new)
        if not done:
            with np.errstate(divide="ignore", invalid="ignore"):
                self.setCurrRate(float(np.float64(step_mass) / (np.float64(nSteps) * scene.dt)))

    def _box_global(self):
        return None

    def _existing_spheres(self, field):
        """Centres and radii of the spheres in the field that reach into the inlet's box
        (squaredExteriorDistance(pos) <= r^2); every sphere when the inlet has no box."""
        arr = field._arrays
        if arr is not None:
            if field._stale:
                field._engine._download_particles(field)
            live = np.ones(arr.n, bool)
            if field._dead:
                live[list(field._dead)] = False
            ids = np.nonzero(live & (arr.shape == dem.abi.SHAPE_SPHERE))[0]
            C, R = arr.pos[ids].copy(), arr.radius[ids].copy()
        else:
            sph = [p for p in field.par if isinstance(p.shape, dem.Sphere)]
            C = np.array([p.pos for p in sph], np.float64).reshape(-1, 3)
            R = np.array([p.shape.radius for p in sph], np.float64)
        box = self._box_global()
        if box is not None and len(R):
            lo, hi = box
            d = np.maximum(lo[None, :] - C, 0.) + np.maximum(C - hi[None, :], 0.)
            keep = ~(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2] > R * R)
            C, R = C[keep], R[keep]
        return C, R


class BoxInlet(RandomInlet):
    """BoxInlet (Inlet.hpp:243-268, Inlet.cpp:518-525): random positions in the axis-aligned box shrunk by
    padDist; a particle's box must lie in the box."""
    _defaults = dict(box=((nan, nan, nan), (nan, nan, nan)), node=None)

    def _check(self):
        super()._check()
        if self.node is not None:
            raise RuntimeError("BoxInlet.node is not supported (give the box in global coordinates)")

    def _lohi(self):
        lo, hi = self.box
        return np.asarray(lo, np.float64).reshape(3), np.asarray(hi, np.float64).reshape(3)

    def _box_global(self):
        return self._lohi()

    def randomPosition(self, diam, padDist):
        lo, hi = self._lohi()
        lo2, hi2 = lo + padDist, hi - padDist
        return np.array([lo2[k] + (hi2[k] - lo2[k]) * self._rng.random() for k in range(3)])

    def validateBox(self, b):
        return _box_contains_box(self._lohi(), b)


def _loc2glob(node, p):
    from .outlet import rotation_matrix
    return rotation_matrix(node.ori) @ np.asarray(p, np.float64) + np.asarray(node.pos, np.float64)


def _corners(b):
    lo, hi = b
    return [np.array([(hi if i & 1 else lo)[0], (hi if i & 2 else lo)[1], (hi if i & 4 else lo)[2]]) for i in range(8)]


class BoxInlet2d(BoxInlet):
    """BoxInlet2d (Inlet.hpp:290-298): a particle's box must lie in the inlet's box in the plane normal
    to `axis` only (it may stick out along the axis)."""
    _defaults = dict(axis=2)

    def validateBox(self, b):
        a1, a2 = (self.axis + 1) % 3, (self.axis + 2) % 3
        (lo, hi), (blo, bhi) = self._lohi(), b
        return bool(lo[a1] <= blo[a1] and lo[a2] <= blo[a2] and bhi[a1] <= hi[a1] and bhi[a2] <= hi[a2])


class CylinderInlet(RandomInlet):
    """CylinderInlet (Inlet.hpp:271-288, Inlet.cpp:564-590): a cylinder of `radius` along the local x-axis
    of node, x from 0 to `height`; positions uniform in it (shrunk by padDist), every corner of a
    particle's box inside."""
    _defaults = dict(node=None, height=nan, radius=nan)

    def _check(self):
        super()._check()
        if self.node is None:
            raise RuntimeError("CylinderInlet.node==None.")

    def randomPosition(self, diam, padDist):
        if padDist > self.radius:
            raise RuntimeError(f"CylinderInlet.randomPosition: padDist={padDist} > radius={self.radius}")
        r3 = [self._rng.random() for _ in range(3)]
        t = 2 * math.pi * r3[0]
        u = 2 * r3[1]
        r = 2. - u if u > 1. else u
        h = r3[2] * (self.height - 2 * padDist) + padDist
        return _loc2glob(self.node, [h, (self.radius - padDist) * r * math.cos(t), (self.radius - padDist) * r * math.sin(t)])

    def validateBox(self, b):
        from .outlet import glob2loc
        for c in _corners(b):
            p = glob2loc(self.node, c)
            if p[0] < 0. or p[0] > self.height:
                return False
            if p[1] * p[1] + p[2] * p[2] > self.radius * self.radius:
                return False
        return True


class ArcInlet(RandomInlet):
    """ArcInlet (Inlet.hpp:300-315, Inlet.cpp:593-612): positions uniform (in cartesian space) in a box
    of cylindrical coordinates of node's frame, padded by padDist (padDist/rho0 in the angle); every
    corner of a particle's box inside."""
    _defaults = dict(node=None, cylBox=((0., 0., 0.), (0., 0., 0.)))

    def _check(self):
        super()._check()
        if self.node is None:
            raise RuntimeError("ArcInlet.node: must not be None.")
        lo, hi = self.cylBox
        if lo[0] < 0 or hi[0] < 0:
            raise RuntimeError(f"ArcInlet.cylBox: radius bounds (x-component) must be non-negative (not {lo[0]}..{hi[0]}).")

    def randomPosition(self, diam, padDist):
        from .outlet import cyl2cart
        lo, hi = (np.asarray(x, np.float64) for x in self.cylBox)
        pad = np.array([padDist, padDist / lo[0], padDist])
        lo, hi = lo + pad, hi - pad
        rx, ry, rz = (self._rng.random() for _ in range(3))
        # CompUtils::cylCoordBox_sample_cylindrical (CompUtils.cpp:134-143)
        r = math.sqrt(lo[0] * lo[0] + rx * (hi[0] * hi[0] - lo[0] * lo[0]))
        return _loc2glob(self.node, cyl2cart([r, lo[1] + ry * (hi[1] - lo[1]), lo[2] + rz * (hi[2] - lo[2])]))

    def validateBox(self, b):
        from .outlet import cyl_box_contains, glob2loc
        return all(cyl_box_contains(self.cylBox, glob2loc(self.node, c)) for c in _corners(b))
