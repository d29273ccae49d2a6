"""Woo's DEM surface (woo.dem): materials, shapes, particles, contacts, DemField, the functor and
engine classes of the hot path, and GpuDemEngine, the one engine that runs them on the GPU.

Names and attribute defaults follow the reference classes (cited per class).  The objects hold
attributes only; the computation is libwdem.so (no CPU path).  Once a scene has run, particle state
lives on the GPU: reading an attribute downloads the field's state once (bulk), writing one marks the
field so the next run uploads the kinematic state again.
"""
import math

import numpy as np

from . import abi

nan = float("nan")


def _vec3(v):
    a = np.asarray(v, dtype=np.float64).reshape(3)
    return a.copy()


def _quat(q):
    a = np.asarray(q, dtype=np.float64).reshape(4)
    return a.copy()


class _Attrs:
    """Keyword constructor with defaults from a class table (like Woo's attribute macros)."""
    _defaults = {}

    def __init__(self, **kw):
        for cls in reversed(type(self).__mro__):
            for k, v in getattr(cls, "_defaults", {}).items():
                setattr(self, k, v)
        for k, v in kw.items():
            if not any(k in getattr(c, "_defaults", {}) for c in type(self).__mro__) and k != "label":
                raise AttributeError(f"{type(self).__name__} has no attribute {k!r}")
            setattr(self, k, v)
        if "label" not in kw:
            self.label = ""

    def __repr__(self):
        return f"<{type(self).__name__}>"


# ---------------------------------------------------------------------------------------- materials
class Material(_Attrs):
    """Material (src/dem/Particle.hpp:483): density 1000."""
    _defaults = dict(density=1000.0, id=-1)


class ElastMat(Material):
    """ElastMat (src/dem/FrictMat.hpp:6-16): young 1e9."""
    _defaults = dict(young=1e9)


class FrictMat(ElastMat):
    """FrictMat (src/dem/FrictMat.hpp:18-28): tanPhi .5, ktDivKn .2."""
    _defaults = dict(tanPhi=0.5, ktDivKn=0.2)
    _kind = abi.MAT_FRICT


class HertzMat(FrictMat):
    """HertzMat (src/dem/Hertz.hpp:5-14): surfEnergy 0, alpha 0."""
    _defaults = dict(surfEnergy=0.0, alpha=0.0)
    _kind = abi.MAT_HERTZ


# ---------------------------------------------------------------------------------------- nodes
class DemData:
    """DemData (src/dem/Particle.hpp:189-306): per-node dynamic state and flags."""
    DOF_X, DOF_Y, DOF_Z, DOF_RX, DOF_RY, DOF_RZ = 1, 2, 4, 8, 16, 32
    CLUMP_CLUMPED, CLUMP_CLUMP, ENERGY_SKIP, GRAVITY_SKIP, TRACER_SKIP, DAMPING_SKIP = 64, 128, 256, 512, 1024, 2048

    def __init__(self, node):
        self._node = node

    def _get(self, name):
        return self._node._get(name)

    def _set(self, name, v):
        self._node._set(name, v)

    vel = property(lambda s: s._get("vel"), lambda s, v: s._set("vel", _vec3(v)))
    angVel = property(lambda s: s._get("angVel"), lambda s, v: s._set("angVel", _vec3(v)))
    force = property(lambda s: s._get("force"), lambda s, v: s._set("force", _vec3(v)))
    torque = property(lambda s: s._get("torque"), lambda s, v: s._set("torque", _vec3(v)))
    mass = property(lambda s: float(s._get("mass")), lambda s, v: s._set("mass", float(v)))
    inertia = property(lambda s: s._get("inertia"), lambda s, v: s._set("inertia", _vec3(v)))
    flags = property(lambda s: int(s._get("flags")), lambda s, v: s._set("flags", int(v)))
    angMom = property(lambda s: s._get("angMom"), lambda s, v: s._set("angMom", _vec3(v)))

    @property
    def isAspherical(self):
        i = self.inertia
        return not (i[0] == i[1] and i[1] == i[2])

    @property
    def blocked(self):
        f = self.flags
        return "".join(c for i, c in enumerate("xyzXYZ") if f & (1 << i))

    @blocked.setter
    def blocked(self, dofs):
        f = self.flags & ~63
        for c in dofs:
            f |= 1 << "xyzXYZ".index(c)
        self.flags = f

    def _flag(bit):
        return property(lambda s: bool(s.flags & bit),
                        lambda s, v: setattr(s, "flags", (s.flags | bit) if v else (s.flags & ~bit)))

    gravitySkip = _flag(512)
    dampingSkip = _flag(2048)
    energySkip = _flag(256)
    del _flag

    def isBlockedAll(self):
        return (self.flags & 63) == 63

    @property
    def impose(self):
        return None

    @impose.setter
    def impose(self, v):
        """DemData.impose (prescribed motion applied inside Leapfrog::run, src/dem/Leapfrog.cpp:22,205,
        238-248) is not provided by the GPU engine; setting one is an error rather than being ignored."""
        if v is not None:
            raise RuntimeError(f"DemData.impose ({type(v).__name__}) is not supported by the GPU engine")

    def guessMoving(self):
        """DemData::guessMoving (src/dem/Particle.cpp:638-640): whether the node needs motion integration
        (it has mass and a free DOF, or a velocity)."""
        return (self.mass != 0. and not self.isBlockedAll()) or bool(np.any(self.vel != 0)) or \
            bool(np.any(self.angVel != 0))


class Node:
    """Node (src/core/Field.hpp) with DemData; pos and ori (w, x, y, z)."""

    def __init__(self, pos=(0, 0, 0), ori=(1, 0, 0, 0)):
        self._local = dict(pos=_vec3(pos), ori=_quat(ori), vel=np.zeros(3), angVel=np.zeros(3),
                           force=np.zeros(3), torque=np.zeros(3), mass=0.0, inertia=np.zeros(3), flags=0,
                           angMom=np.full(3, nan))
        self._field = None
        self._idx = -1
        self.dem = DemData(self)

    def _get(self, name):
        if self._field is None:
            return self._local[name].copy() if isinstance(self._local[name], np.ndarray) else self._local[name]
        return self._field._get(self._idx, name)

    def _set(self, name, v):
        if self._field is None:
            self._local[name] = v
        else:
            self._field._set(self._idx, name, v)

    pos = property(lambda s: s._get("pos"), lambda s, v: s._set("pos", _vec3(v)))
    ori = property(lambda s: s._get("ori"), lambda s, v: s._set("ori", _quat(v)))

    def __getstate__(self):
        """Pickled with its current state and unbound (a loaded scene uploads it again)."""
        d = dict(self.__dict__)
        f = self._field
        if f is not None and f._arrays is not None and 0 <= self._idx < f._arrays.n:
            d["_local"] = {k: (getattr(f._arrays, k)[self._idx].copy()
                               if isinstance(getattr(f._arrays, k)[self._idx], np.ndarray)
                               else getattr(f._arrays, k)[self._idx].item()) for k in _FIELD_ARRAY_NAMES}
        d["_field"], d["_idx"] = None, -1
        return d


# ---------------------------------------------------------------------------------------- shapes
DEFAULT_MOVABLE_MASK = 0b0101
DEFAULT_BOUNDARY_MASK = 0b0011
DEFAULT_LONE_MASK = 0b0010


class Shape:
    def __init__(self):
        self.nodes = []


class Sphere(Shape):
    """Sphere (src/dem/Sphere.hpp:10-30); mass/inertia from Sphere::lumpMassInertia (Sphere.cpp:26-33)."""
    _shape = abi.SHAPE_SPHERE

    def __init__(self, radius=nan):
        super().__init__()
        self.radius = float(radius)

    @staticmethod
    def make(center, radius, mat=None, fixed=False, mask=DEFAULT_MOVABLE_MASK, vel=None, wire=False, color=None):
        """woo.utils.sphere / Sphere.make (py/utils.py:153-199)."""
        mat = mat if mat is not None else defaultMaterial()
        sh = Sphere(radius)
        n = Node(pos=center)
        sh.nodes.append(n)
        p = Particle(shape=sh, material=mat, mask=mask)
        r = float(radius)
        m = ((4 / 3.0) * math.pi) * (r * r * r) * mat.density
        n.dem.mass = m
        n.dem.inertia = np.full(3, 0.0 + ((2.0 / 5.0) * m) * (r * r))
        if fixed:
            n.dem.blocked = "xyzXYZ"
        if vel is not None:
            n.dem.vel = vel
        return p


class Wall(Shape):
    """Wall (src/dem/Wall.hpp:13-37): axis-aligned plane; sense -1/0/+1."""
    _shape = abi.SHAPE_WALL

    def __init__(self, axis=0, sense=0):
        super().__init__()
        self.axis = int(axis)
        self.sense = int(sense)

    @staticmethod
    def make(position, axis, sense=0, mat=None, fixed=True, mass=0, mask=DEFAULT_BOUNDARY_MASK, glAB=None, color=None):
        """woo.utils.wall (py/utils.py:245-267)."""
        if not fixed and mass <= 0:
            raise ValueError("Non-fixed wall must have positive mass")
        mat = mat if mat is not None else defaultMaterial()
        sh = Wall(axis, sense)
        pos = np.zeros(3)
        if np.ndim(position) == 0:
            pos[axis] = position
        else:
            pos = _vec3(position)
        n = Node(pos=pos)
        sh.nodes.append(n)
        p = Particle(shape=sh, material=mat, mask=mask)
        n.dem.mass = float(mass)
        if fixed:
            n.dem.blocked = "xyzXYZ"
        return p


class Ellipsoid(Shape):
    """Ellipsoid (src/dem/Ellipsoid.hpp:11-40): semiAxes; mass and inertia from
    Ellipsoid::lumpMassInertia (Ellipsoid.cpp:37-44)."""
    _shape = abi.SHAPE_ELLIPSOID

    def __init__(self, semiAxes=(nan, nan, nan)):
        super().__init__()
        self.semiAxes = _vec3(semiAxes)

    def equivRadius(self):
        return float(np.cbrt(self.semiAxes[0] * self.semiAxes[1] * self.semiAxes[2]))

    def volume(self):
        return (4 / 3.0) * math.pi * float(self.semiAxes[0] * self.semiAxes[1] * self.semiAxes[2])

    @staticmethod
    def make(center, semiAxes, ori=(1, 0, 0, 0), mat=None, fixed=False, mask=DEFAULT_MOVABLE_MASK, vel=None):
        """Ellipsoid.make (py/_monkey/... ; the reference's Shape::make + lumpMassInertia)."""
        from . import scenes
        mat = mat if mat is not None else defaultMaterial()
        sh = Ellipsoid(semiAxes)
        if not np.all(sh.semiAxes > 0):
            raise RuntimeError("Ellipsoid: all semi-principal semiAxes must be positive")
        n = Node(pos=center, ori=ori)
        sh.nodes.append(n)
        p = Particle(shape=sh, material=mat, mask=mask)
        m, inertia = scenes.ellipsoid_mass_inertia(sh.semiAxes[None, :], mat.density)
        n.dem.mass = float(m[0])
        n.dem.inertia = inertia[0]
        if fixed:
            n.dem.blocked = "xyzXYZ"
        if vel is not None:
            n.dem.vel = vel
        return p


class Capsule(Shape):
    """Capsule (src/dem/Capsule.hpp:8-35): a cylinder of length shaft along the node's local x axis with
    hemispherical caps of radius; mass and inertia from Capsule::lumpMassInertia (Capsule.cpp:44-57).  On
    the GPU it is an aspherical shape (FrictMat + IdealElPl) contacting spheres, walls and capsules."""
    _shape = abi.SHAPE_CAPSULE

    def __init__(self, radius=nan, shaft=nan):
        super().__init__()
        self.radius = float(radius)
        self.shaft = float(shaft)

    def volume(self):
        """Capsule::volume (Capsule.cpp:25-27)."""
        r = self.radius
        return (4 / 3.0) * math.pi * (r * r * r) + math.pi * (r * r) * self.shaft

    def equivRadius(self):
        return float(np.cbrt(self.volume() * 3 / (4 * math.pi)))

    def endPt(self, i):
        """Capsule::endPt (Capsule.hpp:24): end 0 at local -shaft/2 x, end 1 at +shaft/2 x."""
        from . import scenes
        n = self.nodes[0]
        return n.pos + scenes.quat_rotate(n.ori, ((-.5 if i == 0 else .5) * self.shaft, 0, 0))

    @staticmethod
    def make(center, radius, shaft, ori=(1, 0, 0, 0), mat=None, fixed=False, mask=DEFAULT_MOVABLE_MASK, wire=False,
             color=None):
        """woo.utils.capsule / Capsule.make (py/utils.py:213-221)."""
        from . import scenes
        if not (radius > 0) or not (shaft >= 0):
            raise RuntimeError("Capsule: radius must be positive and shaft non-negative")
        mat = mat if mat is not None else defaultMaterial()
        sh = Capsule(radius, shaft)
        n = Node(pos=center, ori=ori)
        sh.nodes.append(n)
        p = Particle(shape=sh, material=mat, mask=mask)
        m, inertia = scenes.capsule_mass_inertia(radius, shaft, mat.density)
        n.dem.mass = float(m)
        n.dem.inertia = np.asarray(inertia, float)
        if fixed:
            n.dem.blocked = "xyzXYZ"
        return p


class Facet(Shape):
    """Facet (src/dem/Facet.hpp:8-57): a triangle of three nodes with halfThick.  The GPU engine takes fixed
    facets (all DOFs blocked, at rest) without fakeVel and without neighbour angles (n21lim NaN); it contacts
    spheres through Cg2_Facet_Sphere_L6Geom.  The engine binds node 0 to the particle's slot; nodes 1 and 2
    keep their positions."""
    _shape = abi.SHAPE_FACET

    def __init__(self, halfThick=0.0):
        super().__init__()
        self.halfThick = float(halfThick)
        self.fakeVel = np.zeros(3)

    def _verts(self):
        return [nd.pos if k == 0 else nd._local["pos"] for k, nd in enumerate(self.nodes)]

    def getNormal(self):
        """Facet::getNormal (Facet.cpp:74-77): (n1 - n0) x (n2 - n0), normalised."""
        a, b, c = self._verts()
        v = np.cross(b - a, c - a)
        return v / np.linalg.norm(v)

    def getArea(self):
        a, b, c = self._verts()
        return 0.5 * float(np.linalg.norm(np.cross(b - a, c - a)))

    def getCentroid(self):
        a, b, c = self._verts()
        return (a + b + c) / 3.0

    def equivRadius(self):
        return nan

    @staticmethod
    def make(vertices, halfThick=0.0, mat=None, fixed=True, mask=DEFAULT_BOUNDARY_MASK, fakeVel=None, wire=True,
             color=None):
        """woo.utils.facet / Facet.make (py/utils.py:315-341): three new nodes (masses and inertia 0,
        all DOFs blocked when fixed), DemField.defaultBoundaryMask."""
        if fakeVel is not None and np.any(np.asarray(fakeVel, float) != 0):
            raise RuntimeError("Facet.fakeVel is not supported by the GPU engine")
        mat = mat if mat is not None else defaultMaterial()
        sh = Facet(halfThick)
        for v in vertices:
            n = Node(pos=v)
            if fixed:
                n.dem.blocked = "xyzXYZ"
            sh.nodes.append(n)
        if len(sh.nodes) != 3:
            raise ValueError("Facet.make needs three vertices")
        return Particle(shape=sh, material=mat, mask=mask)


def defaultMaterial():
    """woo.utils.defaultMaterial (py/utils.py:86-92)."""
    return FrictMat(density=1e3, young=1e7, ktDivKn=0.2, tanPhi=math.tan(0.5))


# ---------------------------------------------------------------------------------------- particles
class Particle:
    """Particle (src/dem/Particle.hpp:60-130) with the uninodal shorthands pos/ori/vel/angVel/f/t."""

    def __init__(self, shape=None, material=None, mask=1):
        self.shape = shape
        self.material = material
        self._mask = int(mask)
        self.id = -1

    def _bound(self):
        if self.shape is None or not self.shape.nodes:
            return None
        return self.shape.nodes[0]._field

    @property
    def mask(self):
        return self._mask

    @mask.setter
    def mask(self, v):
        """Particle.mask; on a running field the new mask reaches the collider at the next run (contacts
        already in the container stay, as in Woo)."""
        self._mask = int(v)
        f = self._bound()
        if f is not None and f.par.exists(self.id) and f.par[self.id] is self:
            f._set_mask(self.id, self._mask)

    def _node(self):
        if not self.shape or len(self.shape.nodes) != 1:
            raise RuntimeError("uninodal particles only")
        return self.shape.nodes[0]

    pos = property(lambda s: s._node().pos, lambda s, v: setattr(s._node(), "pos", v))
    ori = property(lambda s: s._node().ori, lambda s, v: setattr(s._node(), "ori", v))
    vel = property(lambda s: s._node().dem.vel, lambda s, v: setattr(s._node().dem, "vel", v))
    angVel = property(lambda s: s._node().dem.angVel, lambda s, v: setattr(s._node().dem, "angVel", v))
    f = property(lambda s: s._node().dem.force)
    t = property(lambda s: s._node().dem.torque)
    mass = property(lambda s: s._node().dem.mass)
    inertia = property(lambda s: s._node().dem.inertia)
    blocked = property(lambda s: s._node().dem.blocked, lambda s, v: setattr(s._node().dem, "blocked", v))
    impose = property(lambda s: s._node().dem.impose, lambda s, v: setattr(s._node().dem, "impose", v))

    @property
    def nodes(self):
        return self.shape.nodes

    @property
    def Ekt(self):
        v = self.vel
        return 0.5 * self.mass * float(v @ v)

    @property
    def Ekr(self):
        """Rotational kinetic energy, DemData::getEk_any(rot) (src/dem/Particle.cpp:257-263), without
        the periodic cell's spin."""
        from .outlet import kinetic_energy
        return kinetic_energy(0.0, self.inertia, self.pos, self.vel, self.angVel, self.ori, 0.0)

    @property
    def Ek(self):
        return self.Ekt + self.Ekr


class ParticleContainer:
    """S.dem.par (src/dem/ParticleContainer.hpp)."""

    def __init__(self, field):
        self._field = field
        self._list = []
        self._free = []

    def add(self, par, nodes=-1):
        """ParticleContainer.add (pyAppend, ParticleContainer.cpp:176-207): nodes=True puts the particle's
        node into DemField.nodes (integrated by Leapfrog), False leaves it out, -1 decides by
        DemData.guessMoving.  The particle takes the first free id (findFreeId, :23-36): an id left by
        a removed particle, else the next one past the end."""
        if isinstance(par, (list, tuple)):
            ids = [self._add_one(p, nodes) for p in par]
            self._field._particles_added([self._list[i] for i in ids])
            return ids
        i = self._add_one(par, nodes)
        self._field._particles_added([par])
        return i

    def _add_one(self, par, nodes):
        if par is None:
            raise ValueError("Particle to be added is None.")
        if par.id >= 0:
            raise IndexError(f"Particle already has id {par.id} set; appending such particle (for the second time) "
                             "is not allowed.")
        if nodes not in (-1, 0, 1):
            raise ValueError(f"nodes must be in {{-1,0,1}} (not {nodes}).")
        id = len(self._list)
        while self._free:
            f = self._free.pop(0)
            if f <= len(self._list):
                id = f
                break
        node = par.shape.nodes[0]
        par._integrated = bool(nodes) if nodes != -1 else node.dem.guessMoving()
        par.id = id
        if id == len(self._list):
            self._list.append(par)
        else:
            self._list[id] = par
        return par.id

    def __getitem__(self, i):
        """ParticleContainer::pyGetItem (ParticleContainer.cpp:230-235): negative ids count from the end;
        an id without a particle raises IndexError."""
        n = len(self._list)
        if -n <= i < 0:
            i += n
        if not self.exists(i):
            raise IndexError(f"No such particle: #{i}.")
        return self._list[i]

    def __len__(self):
        """Size of the id range (ids of removed particles included, trailing ones trimmed)."""
        return len(self._list)

    def __iter__(self):
        """Existing particles by increasing id (ParticleContainer::pyIterator::next skips removed ids)."""
        return (p for p in self._list if p is not None)

    def exists(self, id):
        return 0 <= id < len(self._list) and self._list[id] is not None

    def remove(self, ids):
        """ParticleContainer.remove (pyRemove / pyRemoveList, ParticleContainer.cpp:107-117): remove one
        particle (returns whether it existed) or a sequence of them (list of such flags), with all of
        their contacts (DemField::removeParticle, Particle.cpp:483-530).  Ids of the other particles do
        not change; a removed id is left empty."""
        if isinstance(ids, (list, tuple, np.ndarray)):
            ids = [int(i) for i in ids]
            done = [self.exists(i) for i in ids]
            gone = sorted({i for i, d in zip(ids, done) if d})
        else:
            ok = self.exists(int(ids))
            gone = [int(ids)] if ok else []
            done = ok
        if gone:
            self._field._remove_particles(gone)
        return done

    def remask(self, ids, mask, visible=True, removeContacts=False, removeOverlapping=False):
        """ParticleContainer.remask (ParticleContainer.cpp:239-273): new mask (and visibility) for the
        particles; with removeContacts, their contacts that may no longer collide (Collider::mayCollide
        under the new masks) are removed.  removeOverlapping tests the collider's bounding boxes, which
        live on the GPU, and is not provided."""
        if removeOverlapping:
            raise RuntimeError("ParticleContainer.remask(removeOverlapping=True) is not supported")
        ids = [int(i) for i in ids]
        for i in ids:
            if not self.exists(i):
                raise IndexError(f"No such particle: #{i}.")
        for i in ids:
            self._list[i].mask = int(mask)
            self._list[i].shape.visible = bool(visible)
        if removeContacts:
            self._field._remove_uncollidable_contacts(ids)

    def disappear(self, ids, mask):
        """remask(ids, mask, visible=False, removeContacts=True)."""
        self.remask(ids, mask, visible=False, removeContacts=True, removeOverlapping=False)

    def reappear(self, ids, mask, removeOverlapping=False):
        """remask(ids, mask, visible=True, removeContacts=False, removeOverlapping)."""
        self.remask(ids, mask, visible=True, removeContacts=False, removeOverlapping=removeOverlapping)

    def _drop(self, ids):
        for i in ids:
            self._list[i] = None
            self._free.append(i)
        # removing the last particle shrinks the container (ParticleContainer::remove, :150-154)
        while self._list and self._list[-1] is None:
            self._list.pop()


# ---------------------------------------------------------------------------------------- contacts
class L6Geom:
    """L6Geom (src/dem/L6Geom.hpp:10-24): trsf rows are... columns are the local axes."""

    def __init__(self, uN, vel, angVel, trsf_cols, contPt, ori, lens, contA):
        self.uN = uN
        self.vel = vel
        self.angVel = angVel
        self.trsf = np.stack([trsf_cols[0:3], trsf_cols[3:6], trsf_cols[6:9]], axis=1)
        self.node = Node(pos=contPt, ori=ori)
        self.lens = lens
        self.contA = contA


class FrictPhys:
    """FrictPhys (src/dem/FrictMat.hpp:30-41); HertzPhys adds kn/kt as current stiffnesses."""

    def __init__(self, force, torque, kn, kt, tanPhi):
        self.force = force
        self.torque = torque
        self.kn = kn
        self.kt = kt
        self.tanPhi = tanPhi


class HertzPhys(FrictPhys):
    pass


class Contact:
    """Contact (src/dem/Contact.hpp:47-121)."""

    def __init__(self, arrays, i, field):
        ca = arrays
        self.id1 = int(ca.idA[i])
        self.id2 = int(ca.idB[i])
        self.real = bool(ca.real[i])
        self.stepCreated = int(ca.stepCreated[i])
        self.minDist00Sq = float(ca.minDist00Sq[i])
        if self.real:
            pa, pb = field.par[self.id1], field.par[self.id2]
            if isinstance(pa.shape, Sphere) and isinstance(pb.shape, Sphere) or \
                    isinstance(pa.shape, Wall) and isinstance(pb.shape, Sphere):
                r1 = -pb.shape.radius if isinstance(pa.shape, Wall) else pa.shape.radius
                r2 = pb.shape.radius
            elif isinstance(pa.shape, Facet):
                # Cg2_Facet_Sphere_L6Geom: max(halfThick, radius) and radius (Facet.cpp:389)
                r1, r2 = max(pa.shape.halfThick, pb.shape.radius), pb.shape.radius
            elif isinstance(pb.shape, Capsule):
                # the capsule functors pass the radii (a wall's as -radius, Capsule.cpp:163, 215, 322)
                r2 = pb.shape.radius
                r1 = -r2 if isinstance(pa.shape, Wall) else pa.shape.radius
            else:
                # ellipsoid functors: distances of the contact point from the centres (Ellipsoid.cpp:250, 349)
                cp = ca.contPt[i]
                r2 = float(np.linalg.norm(cp - pb.pos))
                r1 = -r2 if isinstance(pa.shape, Wall) else float(np.linalg.norm(cp - pa.pos))
            lens = np.array([abs(r1), abs(r2)])
            rr = min(r1, r2) if (r1 > 0 and r2 > 0) else (r1 if r1 > 0 else r2)
            self.geom = L6Geom(float(ca.uN[i]), ca.geomVel[i].copy(), ca.geomAngVel[i].copy(), ca.trsf[i],
                               ca.contPt[i], ca.geomOri[i], lens, math.pi * rr * rr)
            cls = HertzPhys if isinstance(pa.material, HertzMat) and isinstance(pb.material, HertzMat) and \
                field._engine_cp2() == abi.CP2_HERTZ else FrictPhys
            self.phys = cls(ca.force[i].copy(), ca.torque[i].copy(), float(ca.kn[i]), float(ca.kt[i]), float(ca.tanPhi[i]))
        else:
            self.geom = None
            self.phys = None

    @property
    def ids(self):
        return (min(self.id1, self.id2), max(self.id1, self.id2))

    def forceSign(self, p):
        pid = p if isinstance(p, int) else p.id
        if pid not in (self.id1, self.id2):
            raise RuntimeError(f"Contact.forceSign: particle #{pid} does not participate in ##{self.id1}+{self.id2}.")
        return 1 if pid == self.id1 else -1

    def isFresh(self, scene):
        return scene.step == self.stepCreated

    def __repr__(self):
        return f"<Contact ##{self.id1}+{self.id2}>"


class ContactContainer:
    """S.dem.con (src/dem/ContactContainer.hpp:16-140): all contacts by linear index or id pair;
    iteration yields real contacts only."""

    def __init__(self, field):
        self._field = field

    def _arrays(self):
        return self._field._contacts()

    def __len__(self):
        return self._arrays().n

    def __getitem__(self, key):
        ca = self._arrays()
        if isinstance(key, (tuple, list)):
            a, b = min(key), max(key)
            k = (a << 32) | b
            idx = np.nonzero(ca.keys() == k)[0]
            return Contact(ca, int(idx[0]), self._field) if len(idx) else None
        n = ca.n
        if key < -n or key >= n:
            raise IndexError(f"Linear index out of range ({-n}..{n - 1})")
        return Contact(ca, key % n, self._field)

    def __iter__(self):
        ca = self._arrays()
        for i in np.nonzero(ca.real)[0]:
            yield Contact(ca, int(i), self._field)

    def countReal(self):
        return int(self._arrays().real.sum())

    def clear(self):
        """ContactContainer.clear: every contact (real or potential) is removed, history included; the
        collider then runs in full at the next step."""
        f = self._field
        if f._engine is not None:
            f._engine._clear_contacts(f)

    def realRatio(self):
        n = len(self)
        return self.countReal() / n if n else float("nan")

    def exists(self, a, b):
        return self[(a, b)] is not None

    def existsReal(self, a, b):
        c = self[(a, b)]
        return c is not None and c.real


# ---------------------------------------------------------------------------------------- field
_FIELD_ARRAY_NAMES = ("pos", "ori", "vel", "angVel", "force", "torque", "mass", "inertia", "flags", "angMom")


def _bind_nodes(p, field):
    """The particle's node state lives in the field's arrays at its id; a facet binds node 0 only (nodes 1
    and 2 are fixed positions carried in ParticleArrays.facetVerts)."""
    nodes = p.shape.nodes[:1] if isinstance(p.shape, Facet) else p.shape.nodes
    for n in nodes:
        n._field, n._idx = field, p.id


class DemField:
    """DemField (src/dem/Particle.hpp:310-391)."""
    defaultMovableBit, defaultBoundaryBit, defaultOutletBit, defaultStaticBit = 1, 2, 4, 8
    defaultLoneMask, defaultMovableMask, defaultBoundaryMask = 2, 5, 3
    defaultStaticMask, defaultInletMask, defaultOutletMask, defaultHighestBit = 11, 5, 4, 8

    def __init__(self, gravity=(0, 0, 0), distFactor=-1.0, loneMask=DEFAULT_LONE_MASK, par=None):
        self.gravity = _vec3(gravity)
        self.distFactor = float(distFactor)
        self.loneMask = int(loneMask)
        self.par = ParticleContainer(self)
        self.con = ContactContainer(self)
        self.scene = None
        self._engine = None
        self._arrays = None      # abi.ParticleArrays once bound to an engine
        self._stale = False      # device state newer than _arrays
        self._dirty = set()      # host edits not yet uploaded
        self._dead = set()       # slots of removed particles on the device (never collide, never move)
        self._con_cache = None
        if par:
            self.par.add(list(par))

    # --- binding to the engine
    def _engine_bound(self):
        return self._engine is not None

    def _engine_cp2(self):
        return self._engine._cp2_kind if self._engine else abi.CP2_FRICT

    def _bind(self, engine, arrays):
        self._engine = engine
        self._arrays = arrays
        # slots of existing particles whose node is in DemField.nodes (what outlets look at)
        self._moving = np.zeros(arrays.n, bool)
        for p in self.par:
            _bind_nodes(p, self)
            self._moving[p.id] = getattr(p, "_integrated", True)

    def _get(self, idx, name):
        if self._stale:
            self._engine._download_particles(self)
        v = getattr(self._arrays, name)[idx]
        return v.copy() if isinstance(v, np.ndarray) else (float(v) if name == "mass" else int(v))

    def _set(self, idx, name, v):
        if self._stale:
            self._engine._download_particles(self)
        getattr(self._arrays, name)[idx] = v
        self._dirty.add(name)

    def __getstate__(self):
        d = dict(self.__dict__)
        if self._engine is not None:
            d["_saved_contacts"] = self._engine._download_contacts()
        for k in ("_engine", "_arrays", "_moving"):
            d.pop(k, None)
        d["_stale"], d["_dirty"], d["_dead"], d["_con_cache"] = False, set(), set(), None
        return d

    def __setstate__(self, d):
        self.__dict__.update(d)
        self._engine, self._arrays = None, None

    def _set_mask(self, idx, mask):
        self._arrays.mask[idx] = mask
        self._dirty.add("mask")

    def _particles_added(self, pars):
        """Particles added to a running field reach the GPU at the next run (with the contact history
        of the others), in the slots of their ids."""
        if self._engine is not None:
            self._engine._add_particles(self, pars)

    def _remove_uncollidable_contacts(self, ids):
        """Remove the contacts of the given particles whose pair may no longer collide (mask & mask == 0,
        or a common loneMask bit; Collider::mayCollide, src/dem/Collision.cpp:21-43)."""
        if self._engine is None:
            return
        self._engine._remove_contacts_where(self, ids, self._may_collide)

    def _may_collide(self, a, b):
        ma, mb = self.par[a].mask, self.par[b].mask
        return (ma & mb) != 0 and (ma & mb & self.loneMask) == 0

    def _remove_particles(self, ids):
        """DemField::removeParticle for each id (src/dem/Particle.cpp:483-530): its contacts go, the other
        particles keep their ids and contact history."""
        if self._engine is not None:
            self._engine._remove_particles(self, ids)
            # the removed particles keep their last state, detached from the field
            for i in ids:
                node = self.par._list[i].shape.nodes[0]
                node._local = {k: (getattr(self._arrays, k)[i].copy() if isinstance(getattr(self._arrays, k)[i], np.ndarray)
                                   else getattr(self._arrays, k)[i].item()) for k in _FIELD_ARRAY_NAMES}
                node._field, node._idx = None, -1
        self.par._drop(ids)

    def _contacts(self):
        if self._engine is None:
            return abi.ContactArrays(0)
        if self._con_cache is None:
            self._con_cache = self._engine._download_contacts()
        return self._con_cache

    # --- Woo API
    @property
    def nodes(self):
        """DemField.nodes: the nodes Leapfrog integrates, those added with nodes=True or guessed moving
        (ParticleContainer.add, DemData.guessMoving); fixed particles' nodes are not in it."""
        return [p.shape.nodes[0] for p in self.par if getattr(p, "_integrated", True)]

    def unbalancedForce(self, useMaxForce=False):
        """DemFuncs::unbalancedForce (src/dem/Funcs.cpp:231-258): the mean (or maximum) force norm on the
        moving nodes with no blocked DOF, over the mean force norm of the contacts.  The reference reads
        Contact.phys of every contact in the container; here the mean is over the real contacts (the
        potential ones have no phys)."""
        if self._engine is not None and self._stale:
            self._engine._download_particles(self)
        sumF, maxF, nb = 0., 0., 0
        for p in self.par:
            if not getattr(p, "_integrated", True):
                continue
            d = p.shape.nodes[0].dem
            if d.flags & 63 or d.flags & DemData.CLUMP_CLUMPED:
                continue
            f = d.force
            cur = math.sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2])
            maxF = max(cur, maxF)
            sumF += cur
            nb += 1
        meanF = float(np.float64(sumF) / np.float64(nb)) if nb else float("nan")
        ca = self._contacts()
        sumC, nc = 0., 0
        for i in np.nonzero(ca.real)[0]:
            f = ca.force[i]
            sumC += math.sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2])
            nc += 1
        with np.errstate(divide="ignore", invalid="ignore"):
            meanC = np.float64(sumC) / np.float64(nc)
            return float(np.float64(maxF if useMaxForce else meanF) / meanC)

    def critDt(self):
        """DemField::critDt -> DemFuncs::pWaveDt (src/dem/Particle.cpp:399-404, src/dem/Funcs.cpp:151-175)."""
        dt = math.inf
        for p in self.par:
            if not isinstance(p.material, ElastMat):
                continue
            if isinstance(p.shape, (Sphere, Capsule)):
                r = p.shape.radius
            elif isinstance(p.shape, Ellipsoid):
                r = float(np.min(p.shape.semiAxes))
            else:
                continue
            dt = min(dt, r / (1.0 * math.sqrt(p.material.young / p.material.density)))
        return dt

    @staticmethod
    def minimalEngines(**kw):
        from . import utils
        return utils.defaultEngines(**kw)

    @staticmethod
    def sceneHasField(scene):
        return any(isinstance(f, DemField) for f in scene.fields)


# ---------------------------------------------------------------------------------------- functors
class Functor(_Attrs):
    pass


class BoundFunctor(Functor):
    pass


class Bo1_Sphere_Aabb(BoundFunctor):
    """Bo1_Sphere_Aabb (src/dem/Sphere.hpp:33-42)."""


class Bo1_Wall_Aabb(BoundFunctor):
    """Bo1_Wall_Aabb (src/dem/Wall.cpp:25-38)."""


class CGeomFunctor(Functor):
    pass


class Cg2_Any_Any_L6Geom__Base(CGeomFunctor):
    """Cg2_Any_Any_L6Geom__Base (src/dem/L6Geom.hpp:28-49)."""
    _defaults = dict(noRatch=False, iniLensTouch=True, trsfRenorm=100, approxMask=0)


class Cg2_Sphere_Sphere_L6Geom(Cg2_Any_Any_L6Geom__Base):
    """Cg2_Sphere_Sphere_L6Geom (src/dem/Sphere.cpp:86-117)."""


class Cg2_Wall_Sphere_L6Geom(Cg2_Any_Any_L6Geom__Base):
    """Cg2_Wall_Sphere_L6Geom (src/dem/Wall.cpp:50-84)."""


class Bo1_Capsule_Aabb(BoundFunctor):
    """Bo1_Capsule_Aabb (src/dem/Capsule.hpp:36-46)."""


class Cg2_Sphere_Capsule_L6Geom(Cg2_Any_Any_L6Geom__Base):
    """Cg2_Sphere_Capsule_L6Geom (src/dem/Capsule.cpp:198-216)."""


class Cg2_Wall_Capsule_L6Geom(Cg2_Any_Any_L6Geom__Base):
    """Cg2_Wall_Capsule_L6Geom (src/dem/Capsule.cpp:116-164)."""


class Cg2_Capsule_Capsule_L6Geom(Cg2_Any_Any_L6Geom__Base):
    """Cg2_Capsule_Capsule_L6Geom (src/dem/Capsule.cpp:223-323)."""


class Bo1_Facet_Aabb(BoundFunctor):
    """Bo1_Facet_Aabb (src/dem/Facet.hpp:58-64)."""


class Cg2_Facet_Sphere_L6Geom(Cg2_Any_Any_L6Geom__Base):
    """Cg2_Facet_Sphere_L6Geom (src/dem/Facet.cpp:333-390)."""


class Bo1_Ellipsoid_Aabb(BoundFunctor):
    """Bo1_Ellipsoid_Aabb (src/dem/Ellipsoid.hpp:44-51)."""


class Cg2_Ellipsoid_Ellipsoid_L6Geom(Cg2_Any_Any_L6Geom__Base):
    """Cg2_Ellipsoid_Ellipsoid_L6Geom (src/dem/Ellipsoid.hpp:52-62): brent, brentBits.  brent=False selects
    the Newton solve (unimplemented in the reference), converged to newtonTol, started from warmStart
    'cold' | 'history' | 'mlp' (warmStartWeights: the learned network's WDEM_WARM_NPARAM weights), falling
    back to the cold start after fallbackIters iterations."""
    _defaults = dict(brent=True, brentBits=32, newtonTol=1e-10, warmStart="cold", fallbackIters=4,
                     warmStartWeights=None)


class Cg2_Sphere_Ellipsoid_L6Geom(Cg2_Ellipsoid_Ellipsoid_L6Geom):
    """Cg2_Sphere_Ellipsoid_L6Geom (src/dem/Ellipsoid.hpp:64-72)."""


class Cg2_Wall_Ellipsoid_L6Geom(Cg2_Any_Any_L6Geom__Base):
    """Cg2_Wall_Ellipsoid_L6Geom (src/dem/Ellipsoid.hpp:74-81)."""


class CPhysFunctor(Functor):
    pass


class Cp2_FrictMat_FrictPhys(CPhysFunctor):
    """Cp2_FrictMat_FrictPhys (src/dem/FrictMat.cpp:20-44); tanPhi MatchMaker unset -> min."""
    _defaults = dict(tanPhi=None)


class Cp2_HertzMat_HertzPhys(Cp2_FrictMat_FrictPhys):
    """Cp2_HertzMat_HertzPhys (src/dem/Hertz.hpp:52-62)."""
    _defaults = dict(poisson=0.2, en=nan)


class LawFunctor(Functor):
    pass


class Law2_L6Geom_FrictPhys_IdealElPl(LawFunctor):
    """Law2_L6Geom_FrictPhys_IdealElPl (src/dem/IdealElPl.hpp:6-28)."""
    _defaults = dict(iniEqlb=False, relRollStiff=0.0, relTwistStiff=0.0, rollTanPhi=0.0, noSlip=False,
                     noBreak=False, noFrict=False)


class Law2_L6Geom_HertzPhys_DMT(LawFunctor):
    """Law2_L6Geom_HertzPhys_DMT (src/dem/Hertz.hpp:67-101)."""
    _defaults = dict(noAttraction=True)


# ---------------------------------------------------------------------------------------- engines
class Master:
    """woo.master: timingEnabled switches engine timing on (Master.timingEnabled, Engine.execTime and
    Engine.execCount, src/core/Engine.hpp:92-94)."""

    def __init__(self):
        self.timingEnabled = False


master = Master()


class Engine(_Attrs):
    """Engine (src/core/Engine.hpp:19-104): dead; execTime (ns) and execCount, accumulated while
    master.timingEnabled is set."""
    _defaults = dict(dead=False, execTime=0, execCount=0)

    def critDt(self):
        return math.inf


class PeriodicEngine(Engine):
    """PeriodicEngine (src/core/Engine.hpp:129-161) for engines that run on the host between GPU steps.
    Activation follows PeriodicEngine::isActivated (src/core/Engine.cpp:170-195) with the step
    criterion; virtPeriod and realPeriod (simulation and wall-clock time) are not supported, since the
    GPU runs the steps between two activations without stopping."""
    _defaults = dict(virtPeriod=0.0, realPeriod=0.0, stepPeriod=1, stepModulo=True, nDo=-1, nDone=0,
                     initRun=True, virtLast=nan, realLast=nan, stepLast=-1, stepPrev=-1, virtPrev=-1.0,
                     realPrev=-1.0)

    def _check(self):
        if self.virtPeriod > 0 or self.realPeriod > 0:
            raise RuntimeError(f"{type(self).__name__}: virtPeriod/realPeriod are not supported on the GPU engine "
                               "(use stepPeriod)")

    def _exhausted(self):
        return self.stepPeriod <= 0 or (self.nDo >= 0 and self.nDone >= self.nDo)

    def _next_step(self, s, time):
        """The first step >= s at which isActivated may fire (None: never), given that it is evaluated in
        every step from s on (a dead engine is not evaluated).  The first evaluation starts the count
        (Engine.cpp:175-178); where it does not fire, that is all it does, so it is done here."""
        if self.dead:
            return None
        per = int(self.stepPeriod)
        if self.stepLast < 0:
            if not self._exhausted() and self.stepModulo and s % per == 0:
                return s
            self.stepLast = s
            self.virtLast = time
            self.realLast = _clock()
        if self._exhausted():
            return None
        t = self.stepLast + per
        if self.stepModulo:
            t = min(t, -(-s // per) * per)
        return max(t, s)

    def _activate(self, s, time):
        """PeriodicEngine::isActivated at step s (Engine.cpp:170-195), step criterion."""
        now = _clock()
        init = self.stepLast < 0
        if init:
            self.realLast, self.virtLast, self.stepLast = now, time, s
        per = int(self.stepPeriod)
        if (self.nDo < 0 or self.nDone < self.nDo) and per > 0 and \
                ((s - self.stepLast >= per) or (self.stepModulo and s % per == 0)):
            self.realPrev, self.realLast = self.realLast, now
            self.virtPrev, self.virtLast = self.virtLast, time
            self.stepPrev, self.stepLast = self.stepLast, s
            if init and not self.initRun:
                return False
            self.nDone += 1
            return True
        return False

    def run(self, scene):
        raise NotImplementedError


def _clock():
    import time as _t
    return _t.time()


class Leapfrog(Engine):
    """Leapfrog (src/dem/Leapfrog.hpp:17-61)."""
    _defaults = dict(damping=0.2, reset=False, kinSplit=False, dontCollect=False)


class InsertionSortCollider(Engine):
    """InsertionSortCollider (src/dem/InsertionSortCollider.hpp:264-296) + AabbCollider.verletDist."""
    _defaults = dict(verletDist=-0.05, sortAxis=0, forceInitSort=False, sortThenCollide=False)

    def __init__(self, boundFunctors=None, **kw):
        super().__init__(**kw)
        self.boundFunctors = list(boundFunctors or [])


class ContactLoop(Engine):
    """ContactLoop (src/dem/ContactLoop.hpp:110-130); constructed from 3 functor lists."""
    _defaults = dict(applyForces=True, updatePhys="never", dist00=True, evalStress=False, reorderEvery=1000)

    def __init__(self, cg2=None, cp2=None, law=None, **kw):
        super().__init__(**kw)
        self.geoFunctors = list(cg2 or [])
        self.phyFunctors = list(cp2 or [])
        self.lawFunctors = list(law or [])


class DynDt(Engine):
    """DynDt (src/dem/DynDt.hpp:5-27): adjusts Scene.dt from the contact stiffnesses every stepPeriod
    steps (a PeriodicEngine with stepModulo); run by the GPU engine after its contact pass (sphere and
    wall scenes).  dryRun is not provided."""
    _defaults = dict(stepPeriod=100, maxRelInc=1e-4, dryRun=False)


_UPDATE_PHYS = {"never": abi.UPDATE_PHYS_NEVER, "always": abi.UPDATE_PHYS_ALWAYS, "once": abi.UPDATE_PHYS_ONCE}


class GpuDemEngine(Engine):
    """One GPU engine replacing [Leapfrog, InsertionSortCollider, ContactLoop].

    Constructed like ContactLoop from the three functor lists (src/dem/ContactLoop.cpp:52-66), plus
    the Leapfrog (damping, reset) and collider (verletDist) attributes.  Runs libwdem.so on one CUDA
    device; errors come back as RuntimeError.  arith: "exact" (the reference's IEEE operations, bit for
    bit), "fma" (FP64 multiply-adds contracted, one reciprocal per vector division) or "dw" (as "fma", with
    the contact law of real sphere and wall contacts in double-word FP32).  autotune: pick the
    kernels' launch shape on the first run (woo_gb300.tuning: cached per GPU and workload)."""
    _defaults = dict(capacity=0, damping=0.2, reset=True, kinSplit=False, verletDist=-0.05, applyForces=True,
                     updatePhys="never", dist00=True, device=0, keepGeom=True, arith="exact", autotune=False)

    def __init__(self, cg2=None, cp2=None, law=None, **kw):
        super().__init__(**kw)
        self.geoFunctors = list(cg2 or [Cg2_Sphere_Sphere_L6Geom(), Cg2_Facet_Sphere_L6Geom(), Cg2_Wall_Sphere_L6Geom(),
                                        Cg2_Wall_Capsule_L6Geom(), Cg2_Capsule_Capsule_L6Geom(),
                                        Cg2_Sphere_Capsule_L6Geom()])
        self.phyFunctors = list(cp2 or [Cp2_FrictMat_FrictPhys()])
        self.lawFunctors = list(law or [Law2_L6Geom_FrictPhys_IdealElPl()])
        self._h = None
        self._mats = None
        self._params = None
        self._field = None
        self._cp2_kind = abi.CP2_FRICT

    @classmethod
    def fromEngines(cls, engines):
        """Build from Woo's [Leapfrog, InsertionSortCollider, ContactLoop] (py/utils.py:122-129)."""
        lf = next(e for e in engines if isinstance(e, Leapfrog))
        col = next(e for e in engines if isinstance(e, InsertionSortCollider))
        cl = next(e for e in engines if isinstance(e, ContactLoop))
        g = cls(cl.geoFunctors, cl.phyFunctors, cl.lawFunctors, damping=lf.damping, reset=lf.reset,
                kinSplit=lf.kinSplit, verletDist=col.verletDist, applyForces=cl.applyForces,
                updatePhys=cl.updatePhys, dist00=cl.dist00)
        g.label = cl.label or "gpu"
        g._sources = dict(leapfrog=lf, collider=col, contactLoop=cl)
        return g

    # ------------------------------------------------------------------ functor selection
    def _functor(self, lst, classes):
        for f in lst:
            if isinstance(f, classes):
                return f
        return None

    def _build_params(self, scene, field):
        geo = self._functor(self.geoFunctors, (Cg2_Any_Any_L6Geom__Base,)) or Cg2_Sphere_Sphere_L6Geom()
        if any(isinstance(p.shape, Ellipsoid) for p in field.par) and \
                self._functor(self.geoFunctors, (Cg2_Ellipsoid_Ellipsoid_L6Geom,)) is None:
            raise RuntimeError("ellipsoids in the scene need Cg2_Ellipsoid_Ellipsoid_L6Geom (or its sphere variant) "
                               "in ContactLoop.geoFunctors")
        if any(isinstance(p.shape, Facet) for p in field.par) and \
                self._functor(self.geoFunctors, (Cg2_Facet_Sphere_L6Geom,)) is None:
            raise RuntimeError("facets in the scene need Cg2_Facet_Sphere_L6Geom in ContactLoop.geoFunctors")
        if any(isinstance(p.shape, Capsule) for p in field.par):
            missing = [c.__name__ for c in (Cg2_Sphere_Capsule_L6Geom, Cg2_Wall_Capsule_L6Geom, Cg2_Capsule_Capsule_L6Geom)
                       if self._functor(self.geoFunctors, (c,)) is None]
            if missing:
                raise RuntimeError("capsules in the scene need " + ", ".join(missing) + " in ContactLoop.geoFunctors")
        cp2 = self._functor(self.phyFunctors, (Cp2_HertzMat_HertzPhys,)) or self._functor(self.phyFunctors, (Cp2_FrictMat_FrictPhys,))
        law = self._functor(self.lawFunctors, (Law2_L6Geom_HertzPhys_DMT,)) or self._functor(self.lawFunctors, (Law2_L6Geom_FrictPhys_IdealElPl,))
        if cp2 is None or law is None:
            raise RuntimeError("GpuDemEngine needs a Cp2 (FrictMat/HertzMat) and a Law2 (IdealElPl/HertzPhys_DMT) functor")
        if getattr(cp2, "tanPhi", None) is not None:
            raise RuntimeError("Cp2_FrictMat_FrictPhys.tanPhi MatchMaker is not supported")
        mats = {}
        for p in field.par:
            mats.setdefault(id(p.material), p.material)
        mlist = list(mats.values())
        if isinstance(cp2, Cp2_HertzMat_HertzPhys):
            bad = sorted({type(m).__name__ for m in mlist if not isinstance(m, HertzMat)})
            if bad:
                # ContactLoop.cpp:181: a CPhysFunctor must exist for every contacting material pair, and
                # Cp2_HertzMat_HertzPhys takes HertzMat only (Hertz.hpp:54)
                raise RuntimeError(f"Cp2_HertzMat_HertzPhys needs HertzMat for every particle (found {', '.join(bad)}): "
                                   "a CPhysFunctor must be available for every contacting material combination")
        self._mat_index = {id(m): i for i, m in enumerate(mlist)}
        arr = (abi.Material * len(mlist))()
        for i, m in enumerate(mlist):
            arr[i].kind = getattr(m, "_kind", abi.MAT_FRICT)
            arr[i].density = m.density
            arr[i].young = m.young
            arr[i].ktDivKn = getattr(m, "ktDivKn", 0.2)
            arr[i].tanPhi = getattr(m, "tanPhi", 0.5)
            arr[i].surfEnergy = getattr(m, "surfEnergy", 0.0)
            arr[i].alpha = getattr(m, "alpha", 0.0)
        self._mats = arr
        self._mlist = mlist
        p = abi.Params()
        p.dt = scene.dt
        p.step = scene.step
        for k in range(3):
            p.gravity[k] = field.gravity[k]
        p.distFactor = field.distFactor
        p.loneMask = field.loneMask
        p.trackEnergy = 1 if scene.trackEnergy else 0
        p.damping = self.damping
        p.reset = 1 if self.reset else 0
        p.kinSplit = 1 if self.kinSplit else 0
        p.verletDist = self.verletDist
        p.noRatch = int(geo.noRatch); p.iniLensTouch = int(geo.iniLensTouch)
        p.trsfRenorm = int(geo.trsfRenorm); p.approxMask = int(geo.approxMask)
        p.updatePhys = _UPDATE_PHYS[self.updatePhys] if isinstance(self.updatePhys, str) else int(self.updatePhys)
        p.applyForces = int(self.applyForces)
        p.dist00 = int(self.dist00)
        if isinstance(cp2, Cp2_HertzMat_HertzPhys):
            p.cp2 = abi.CP2_HERTZ; p.poisson = cp2.poisson; p.en = cp2.en
        else:
            p.cp2 = abi.CP2_FRICT; p.poisson = 0.2; p.en = nan
        self._cp2_kind = p.cp2
        if isinstance(law, Law2_L6Geom_HertzPhys_DMT):
            p.law = abi.LAW_HERTZ_DMT; p.noAttraction = int(law.noAttraction)
        else:
            p.law = abi.LAW_IDEALELPL
            p.noSlip = int(law.noSlip); p.noBreak = int(law.noBreak); p.noFrict = int(law.noFrict)
            p.iniEqlb = int(law.iniEqlb)
            p.relRollStiff = law.relRollStiff; p.relTwistStiff = law.relTwistStiff; p.rollTanPhi = law.rollTanPhi
            p.noAttraction = 1
        p.nMaterials = len(mlist)
        p.materials = arr
        ell = self._functor(self.geoFunctors, (Cg2_Ellipsoid_Ellipsoid_L6Geom,))
        p.ellSolver = abi.ELL_BRENT if (ell is None or ell.brent) else abi.ELL_NEWTON
        p.brentBits = int(ell.brentBits) if ell is not None else 32
        p.newtonTol = float(ell.newtonTol) if ell is not None else 1e-10
        p.warmStart = {"cold": abi.WARM_COLD, "history": abi.WARM_HISTORY, "mlp": abi.WARM_MLP,
                       "history+mlp": abi.WARM_HISTORY_MLP}[
            ell.warmStart if ell is not None else "cold"]
        p.fallbackIters = int(ell.fallbackIters) if ell is not None else 4
        if self.arith not in ("exact", "fma", "dw"):
            raise ValueError("GpuDemEngine.arith must be 'exact', 'fma' or 'dw'")
        p.arith = {"exact": abi.ARITH_EXACT, "fma": abi.ARITH_FMA, "dw": abi.ARITH_DW}[self.arith]
        self._ellFunctor = ell
        return p

    def _pack(self, field):
        n = len(field.par)
        pa = abi.ParticleArrays(n)
        live = [p for p in field.par]
        if not live:
            raise RuntimeError("GpuDemEngine: the field has no particles")
        filler = next((p for p in live if isinstance(p.shape, Sphere)), live[0])
        for i in range(n):
            if not field.par.exists(i):
                # an id left by a removed particle: a dead slot holding a copy of a live particle's data,
                # which the device view keeps fixed and out of every contact
                self._pack_one(pa, i, filler)
                field._dead.add(i)
        for p in live:
            self._pack_one(pa, p.id, p)
        return pa

    def _pack_one(self, pa, i, p):
        sh = p.shape
        if isinstance(sh, Sphere):
            pa.shape[i] = abi.SHAPE_SPHERE; pa.radius[i] = sh.radius
        elif isinstance(sh, Wall):
            pa.shape[i] = abi.SHAPE_WALL; pa.wallAxis[i] = sh.axis; pa.wallSense[i] = sh.sense
        elif isinstance(sh, Ellipsoid):
            pa.shape[i] = abi.SHAPE_ELLIPSOID; pa.semiAxes[i] = sh.semiAxes
        elif isinstance(sh, Capsule):
            pa.shape[i] = abi.SHAPE_CAPSULE; pa.radius[i] = sh.radius; pa.shaft[i] = sh.shaft
        elif isinstance(sh, Facet):
            pa.shape[i] = abi.SHAPE_FACET; pa.radius[i] = sh.halfThick
            pa.facetVerts[i] = np.concatenate(sh._verts())
        else:
            raise RuntimeError(f"GpuDemEngine: unsupported shape {type(sh).__name__}")
        pa.material[i] = self._mat_index[id(p.material)]
        pa.mask[i] = p.mask
        node = sh.nodes[0]
        for name in _FIELD_ARRAY_NAMES:
            getattr(pa, name)[i] = node._local[name]

    def _device_view(self, field, pa):
        """The arrays as uploaded: a particle whose node is not in DemField.nodes is never moved by
        Leapfrog, so the GPU engine holds it fixed (all DOFs blocked, no velocity).  The slot of a
        removed particle is held fixed as well and gets mask 0, so that Collider::mayCollide
        (src/dem/Collision.cpp:21-43) never pairs it."""
        idle = [p.id for p in field.par if not getattr(p, "_integrated", True)]
        dead = sorted(field._dead)
        if not idle and not dead:
            return pa
        up = pa.copy()
        for ids in (idle, dead):
            up.flags[ids] |= 63
            up.vel[ids] = 0
            up.angVel[ids] = 0
        if dead:
            up.mask[dead] = 0
            park = self._park_positions(field, pa, dead)
            if park is not None:
                up.pos[dead] = park
        return up

    def _park_positions(self, field, pa, dead):
        """Where the slots `dead` (sorted) are parked: on live spheres, spread over them so that many removed
        particles do not crowd one grid cell, and so that a particle removed far outside the domain does not
        stretch the collider's grid."""
        anchors = [p.id for p in field.par if isinstance(p.shape, Sphere)]
        if not anchors:
            return None
        return pa.pos[np.asarray(anchors)[np.arange(len(dead)) % len(anchors)]]

    def _remove_particles(self, field, ids):
        """Remove particles from a running field, on the device (wdem_remove_particles): their contacts
        leave the container and their slots become dead; the other contacts keep their history and nothing
        but the ids and park positions crosses to the device.  The collider rebuilds at the next step, which
        does not change the motion (every pair that can touch before the next rebuild is found)."""
        if field._stale:
            self._download_particles(field)
        ids = sorted(int(i) for i in ids)
        field._dead.update(ids)
        field._moving[ids] = False
        dead = sorted(field._dead)
        park = self._park_positions(field, field._arrays, dead)
        if park is not None:
            where = {d: k for k, d in enumerate(dead)}
            park = park[[where[i] for i in ids]]
        self._h.remove_particles(ids, park)
        field._con_cache = None

    # ------------------------------------------------------------------ engine protocol
    def critDt(self):
        return math.inf

    def _ensure(self, scene, field):
        if self._h is not None:
            return
        params = self._build_params(scene, field)
        pa = self._pack(field)
        cap = max(pa.n, 1, int(self.capacity))
        inlets = [e for e in getattr(scene, "_host", []) if hasattr(e, "_reserve")]
        if inlets and not self.capacity:
            # room for the particles the inlets may add (their maxNum / maxMass), else twice the scene
            res = [e._reserve() for e in inlets]
            cap = max(cap, pa.n + (sum(res) if all(r is not None for r in res) else max(pa.n, 1024)))
        self._cap = cap
        if not hasattr(self, "_energy_base"):
            self._energy_base = {}
        h = abi.Handle(cap, device=self.device)
        h.keep_geom(self.keepGeom)
        h.set_params(params)
        h.upload_particles(self._device_view(field, pa))
        h.set_params(params)
        if getattr(scene, "periodic", False):
            c = scene.cell
            h.set_cell(c.hSize, c.trsf, c.gradV, c.nextGradV)
        ell = getattr(self, "_ellFunctor", None)
        if ell is not None and ell.warmStart in ("mlp", "history+mlp"):
            if ell.warmStartWeights is None:
                raise RuntimeError("Cg2_Ellipsoid_Ellipsoid_L6Geom.warmStart='mlp' needs warmStartWeights")
            h.warm_set_weights(ell.warmStartWeights)
        saved = getattr(field, "_saved_contacts", None)
        if saved is not None:
            # a loaded scene: its contact container, with the history (the collider then runs in full)
            h.upload_contacts(saved)
            field._saved_contacts = None
        self._h, self._params, self._field = h, params, field
        field._bind(self, pa)

    def _refresh_from_sources(self):
        """Attributes set on Woo's trio after the engine was built (S.lab.contactLoop.updatePhys=...)."""
        src = getattr(self, "_sources", None)
        if not src:
            return
        self.damping = src["leapfrog"].damping
        self.updatePhys = src["contactLoop"].updatePhys
        self.dist00 = src["contactLoop"].dist00

    def run(self, scene, nSteps):
        field = scene.dem
        self._refresh_from_sources()
        if self._h is None and next(iter(field.par), None) is None:
            # nothing to integrate yet (an inlet fills the field later): only time advances
            t = scene.time
            for _ in range(int(nSteps)):
                t += scene.dt
            self._time_after = t
            self._ran_time = t - scene.time
            return
        self._ensure(scene, field)
        if field._dirty:
            self._upload_edits(field)
        if self.autotune and not getattr(self, "_tuned", None):
            from . import tuning
            key = tuning.workload_key(len(field.par), self._params.law, getattr(scene, "periodic", False),
                                      any(isinstance(p.shape, (Ellipsoid, Capsule)) for p in field.par))
            self._h.set_params(self._params)

            def probe():
                # a handle with a copy of the state to tune on, so that the run itself does not advance
                if field._stale:
                    self._download_particles(field)
                t = abi.Handle(self._cap, device=self.device)
                t.keep_geom(False)
                t.set_params(self._params)
                t.upload_particles(self._device_view(field, field._arrays))
                t.set_params(self._params)
                if getattr(scene, "periodic", False):
                    c = scene.cell
                    t.set_cell(c.hSize, c.trsf, c.gradV, c.nextGradV)
                con = self._download_contacts()
                if con.n:
                    t.upload_contacts(con)
                return t
            self._tuned = tuning.tuned(self._h, self.device, key, probe=probe)
        p = self._params
        p.dt = scene.dt
        p.step = scene.step
        p.damping = self.damping
        for k in range(3):
            p.gravity[k] = field.gravity[k]
        up = _UPDATE_PHYS[self.updatePhys] if isinstance(self.updatePhys, str) else int(self.updatePhys)
        p.updatePhys = up
        for i, m in enumerate(self._mlist):
            self._mats[i].young = m.young
            self._mats[i].density = m.density
            self._mats[i].tanPhi = getattr(m, "tanPhi", 0.5)
            self._mats[i].ktDivKn = getattr(m, "ktDivKn", 0.2)
        self._h.set_params(p)
        field._stale = True
        field._con_cache = None
        if getattr(scene, "periodic", False):
            c = scene.cell
            if c._edited:
                self._h.set_cell(c.hSize, c.trsf, c.gradV, c.nextGradV)
                c._edited = False
        dyn = getattr(self, "_dynDt", None)
        if dyn is not None and dyn.dryRun:
            raise RuntimeError("DynDt.dryRun is not supported by the GPU engine")
        p.dynDtPeriod = int(dyn.stepPeriod) if dyn is not None else 0
        p.dynDtMaxRelInc = float(dyn.maxRelInc) if dyn is not None else 1e-4
        p.dtSafety = float(scene.dtSafety)
        if dyn is not None:
            self._h.set_params(p)
        timing = bool(master.timingEnabled)
        if timing != getattr(self, "_timing_on", False):
            self._h.set_timing(timing)
            self._timing_on = timing
        t0 = self._h.status().timeSum
        self._h.step(nSteps)
        if timing:
            self._book_times(nSteps)
        st = self._h.status()
        if dyn is None:
            # dt was constant: Scene.time advances by dt per step, as Scene::doOneStep adds it
            t = scene.time
            for _ in range(int(nSteps)):
                t += p.dt
            self._time_after = t
        else:
            self._time_after = scene.time + (st.timeSum - t0)
        self._ran_time = self._time_after - scene.time
        scene.dt = st.dt
        if getattr(scene, "periodic", False):
            cc = self._h.cell()
            scene.cell._sync(cc)
        if up == abi.UPDATE_PHYS_ONCE:
            self.updatePhys = "never"
            if getattr(self, "_sources", None):
                self._sources["contactLoop"].updatePhys = "never"

    def __getstate__(self):
        d = dict(self.__dict__)
        if self._h is not None:
            base = dict(getattr(self, "_energy_base", {}))
            for k, v in self._h.energy().items():
                if k not in ("kinetic", "elast"):
                    base[k] = base.get(k, 0.0) + v
            d["_energy_base"] = base
        for k in ("_h", "_params", "_mats", "_mlist", "_mat_index", "_field", "_timing_on", "_ellFunctor"):
            d.pop(k, None)
        d["_h"] = None
        return d

    def _book_times(self, nSteps):
        """Device time of the three phases (CUDA events around each kernel) as execTime/execCount of this
        engine and of the Leapfrog, InsertionSortCollider and ContactLoop it stands for."""
        kt = self._h.kernel_times()
        self.execTime += int(round(sum(ms for ms, _ in kt.values()) * 1e6))
        self.execCount += nSteps
        src = getattr(self, "_sources", None)
        if src:
            for phase, key in (("leapfrog", "leapfrog"), ("collider", "collider"), ("contacts", "contactLoop")):
                if phase in kt:
                    src[key].execTime += int(round(kt[phase][0] * 1e6))
                    src[key].execCount += nSteps

    def _upload_edits(self, field):
        pa = field._arrays
        n = pa.n
        kin = {"pos", "vel", "angVel", "ori"}
        dv = self._device_view(field, pa)
        added = sorted(getattr(field, "_added", ()))
        # facets (multi-node) are not inserted in place: a full upload takes them
        inplace = not any(isinstance(field.par[i].shape, Facet) for i in added if field.par.exists(i))
        if added and inplace and field._dirty <= kin | {"added"} and n <= self._cap:
            # particles from inlets go into their slots on the device (wdem_add_particles); the rest of
            # the particle and contact state stays there
            self._h.set_params(self._params)   # materials of added particles first
            self._h.add_particles(dv.take(added), added)
            if field._dirty & kin:
                self._h.write_state(n, dv.pos.ctypes.data, dv.vel.ctypes.data, dv.angVel.ctypes.data, dv.ori.ctypes.data)
        elif field._dirty <= kin:
            self._h.write_state(n, dv.pos.ctypes.data, dv.vel.ctypes.data, dv.angVel.ctypes.data, dv.ori.ctypes.data)
        else:
            # mass/inertia/flags/masks changed or particles added: full upload, keeping the contact history
            con = self._download_contacts()
            if n > self._cap:
                self._regrow(field, max(n, 2 * self._cap))
            self._h.set_params(self._params)   # materials of added particles first
            self._h.upload_particles(dv)
            self._h.set_params(self._params)
            self._h.upload_contacts(con)
        field._dirty.clear()
        field._added = set()

    def _remove_contacts_where(self, field, ids, may_collide):
        """Drop the contacts of `ids` for which may_collide(idA, idB) is false; the others keep their
        history.  The particle arrays (with the new masks) and the contacts are uploaded again."""
        if field._stale:
            self._download_particles(field)
        con = self._download_contacts()
        sel = np.isin(con.idA, ids) | np.isin(con.idB, ids)
        drop = np.zeros(con.n, bool)
        for k in np.nonzero(sel)[0]:
            drop[k] = not may_collide(int(con.idA[k]), int(con.idB[k]))
        if drop.any() or field._dirty:
            self._h.set_params(self._params)
            self._h.upload_particles(self._device_view(field, field._arrays))
            self._h.set_params(self._params)
            self._h.upload_contacts(con.take(~drop))
            field._dirty.clear()
        field._con_cache = None

    def _clear_contacts(self, field):
        """An empty contact container replaces the device's (nothing is downloaded).  The particle arrays
        go up with it: they carry the forces of the last contact pass, which the next integration uses as
        Woo's DemData.force outlives the cleared contacts."""
        if field._stale:
            self._download_particles(field)
        self._h.set_params(self._params)
        self._h.upload_particles(self._device_view(field, field._arrays))
        self._h.set_params(self._params)
        self._h.upload_contacts(abi.ContactArrays(0))
        field._dirty.clear()
        field._con_cache = None

    def _add_particles(self, field, pars):
        """Particles added to the running field: packed into the slots of their ids (reused ids of removed
        particles first, as ParticleContainer::findFreeId), uploaded at the next run."""
        if field._stale:
            self._download_particles(field)
        pa = field._arrays
        n = len(field.par)
        if n > pa.n:
            grown = abi.ParticleArrays(n)
            for k, v in pa.__dict__.items():
                if isinstance(v, np.ndarray):
                    getattr(grown, k)[:pa.n] = v
            pa = grown
            field._arrays = pa
            field._moving = np.concatenate([field._moving, np.zeros(n - len(field._moving), bool)])
        for p in pars:
            m = p.material
            if id(m) not in self._mat_index:
                self._add_material(m)
            self._pack_one(pa, p.id, p)
            _bind_nodes(p, field)
            field._dead.discard(p.id)
            field._moving[p.id] = getattr(p, "_integrated", True)
        field._dirty.add("added")
        if not hasattr(field, "_added"):
            field._added = set()
        field._added.update(p.id for p in pars)
        field._con_cache = None

    def _add_material(self, m):
        self._mat_index[id(m)] = len(self._mlist)
        self._mlist.append(m)
        arr = (abi.Material * len(self._mlist))()
        for i in range(len(self._mlist) - 1):
            arr[i] = self._mats[i]
        k = len(self._mlist) - 1
        arr[k].kind = getattr(m, "_kind", abi.MAT_FRICT)
        arr[k].density = m.density
        arr[k].young = m.young
        arr[k].ktDivKn = getattr(m, "ktDivKn", 0.2)
        arr[k].tanPhi = getattr(m, "tanPhi", 0.5)
        arr[k].surfEnergy = getattr(m, "surfEnergy", 0.0)
        arr[k].alpha = getattr(m, "alpha", 0.0)
        self._mats = arr
        self._params.nMaterials = len(self._mlist)
        self._params.materials = arr

    def _regrow(self, field, cap):
        """A new handle with room for `cap` particles, carrying the state over: particles (uploaded by the
        caller), contacts, the periodic cell, and the energies booked so far (kept on the host)."""
        if getattr(self, "_dynDt", None) is not None:
            raise RuntimeError(f"GpuDemEngine: {len(field.par)} particles exceed the engine's capacity {self._cap} "
                               "and DynDt keeps its schedule on the device; set GpuDemEngine.capacity")
        if getattr(field.scene, "periodic", False):
            raise RuntimeError("GpuDemEngine: particles added to a periodic scene beyond the engine's capacity; "
                               "set GpuDemEngine.capacity")
        e = self._h.energy()
        for k, v in e.items():
            # kinetic and elast are reset every step (EnergyTracker::resetResettables): the new handle's value
            # is the current one; the others accumulate
            if k not in ("kinetic", "elast"):
                self._energy_base[k] = self._energy_base.get(k, 0.0) + v
        self._h.close()
        h = abi.Handle(cap, device=self.device)
        h.keep_geom(self.keepGeom)
        self._timing_on = False   # a new handle starts untimed; run() switches it on again if wanted
        ell = getattr(self, "_ellFunctor", None)
        if ell is not None and ell.warmStart in ("mlp", "history+mlp"):
            h.warm_set_weights(ell.warmStartWeights)
        self._h, self._cap = h, cap

    def energy(self):
        """Energies of the run so far (the device's totals plus those of replaced handles)."""
        d = dict(self._h.energy())
        for k, v in getattr(self, "_energy_base", {}).items():
            d[k] = d.get(k, 0.0) + v
        return d

    def _download_particles(self, field):
        self._h.download_particles(field._arrays)
        field._stale = False

    def _download_contacts(self):
        return self._h.download_contacts()

    def status(self):
        return self._h.status() if self._h else None

    def kernelTimes(self):
        return self._h.kernel_times() if self._h else {}


from .outlet import Outlet, BoxOutlet, StackedBoxOutlet, ArcOutlet, CrazyOutlet  # noqa: E402
from .inlet import (Inlet, RandomInlet, BoxInlet, BoxInlet2d, CylinderInlet, ArcInlet,  # noqa: E402
                    ParticleGenerator, MinMaxSphereGenerator, PsdSphereGenerator, AlignedMinMaxShooter)
