"""Seeded synthetic DEM scenes in the engine's SoA format.

Each builder returns a SceneSpec: engine/functor attributes (abi.Params), the materials table and
the particle arrays.  The benchmark scenes follow the configurations the engine is measured on:

* spheres10k   -- 10,000 spheres r=5 mm, FrictMat (rho 3000, E 1e7, ktDivKn .2, tanPhi .5), random
                  sequential addition in a 0.5 x 0.5 x 1.0 m box of 6 walls, gravity -9.81 z,
                  Law2_L6Geom_FrictPhys_IdealElPl, Leapfrog damping .2, dt = 0.4 * p-wave dt.
* hertz1M      -- 1,000,000 spheres r ~ U[2,6] mm, HertzMat E 5e7, tanPhi .3 / .6 (two materials),
                  surfEnergy .01, Cp2_HertzMat_HertzPhys(en=.8), Law2_L6Geom_HertzPhys_DMT, a loose
                  cloud falling into a 1 x 1 x 2 m walled box, dt = 0.3 * p-wave dt,
                  verletDist = 0.1 * rmin.

Masses and inertias follow Sphere::lumpMassInertia (src/dem/Sphere.cpp:26-33).
"""
import ctypes
import math

import numpy as np
from ctypes import c_double as C_double

from . import abi

# The seeded packing generator the builders call: the engine library's (wdem_make_cloud,
# wdem_make_cloud_radii) unless set_packer installs another implementation of the same algorithm.
_PACKER = {"cloud": None, "cloud_radii": None}


def set_packer(cloud=None, cloud_radii=None):
    """Install the functions that build the seeded packings (same signatures as abi.make_cloud and
    abi.make_cloud_radii); None restores the engine library's."""
    _PACKER["cloud"] = cloud
    _PACKER["cloud_radii"] = cloud_radii


def make_cloud(*a, **kw):
    return (_PACKER["cloud"] or abi.make_cloud)(*a, **kw)


def make_cloud_radii(*a, **kw):
    return (_PACKER["cloud_radii"] or abi.make_cloud_radii)(*a, **kw)


# DemField defaults (src/dem/Particle.hpp:334-361)
DEFAULT_MOVABLE_MASK = 0b0101
DEFAULT_BOUNDARY_MASK = 0b0011
DEFAULT_LONE_MASK = 0b0010


class SceneSpec:
    def __init__(self, params, materials, particles, name="", info=None, cell=None):
        self.params = params
        self.materials = materials      # ctypes array kept alive for params.materials
        self.particles = particles
        self.name = name
        self.info = info or {}
        self.cell = cell                # periodic cell: dict(hSize=, trsf=, gradV=, nextGradV=) or None

    def set_dt(self, dt):
        self.params.dt = dt


def materials_array(mats):
    arr = (abi.Material * len(mats))()
    for i, m in enumerate(mats):
        arr[i].kind = m.get("kind", abi.MAT_FRICT)
        arr[i].density = m.get("density", 1000.0)
        arr[i].young = m.get("young", 1e9)
        arr[i].ktDivKn = m.get("ktDivKn", 0.2)
        arr[i].tanPhi = m.get("tanPhi", 0.5)
        arr[i].surfEnergy = m.get("surfEnergy", 0.0)
        arr[i].alpha = m.get("alpha", 0.0)
    return arr


def default_params(materials, **kw):
    """abi.Params with the defaults of Woo's classes (Leapfrog, InsertionSortCollider, ContactLoop,
    Cg2_Any_Any_L6Geom__Base, Cp2/Law2 functors, DemField)."""
    p = abi.Params()
    p.dt = kw.get("dt", float("nan"))
    p.step = kw.get("step", 0)
    g = kw.get("gravity", (0.0, 0.0, 0.0))
    for k in range(3):
        p.gravity[k] = g[k]
    p.distFactor = kw.get("distFactor", -1.0)
    p.loneMask = kw.get("loneMask", DEFAULT_LONE_MASK)
    p.trackEnergy = kw.get("trackEnergy", 0)
    p.damping = kw.get("damping", 0.2)
    p.reset = 1
    p.kinSplit = 0
    p.verletDist = kw.get("verletDist", -0.05)
    p.noRatch = kw.get("noRatch", 0)
    p.iniLensTouch = 1
    p.trsfRenorm = kw.get("trsfRenorm", 100)
    p.approxMask = kw.get("approxMask", 0)
    p.updatePhys = kw.get("updatePhys", abi.UPDATE_PHYS_NEVER)
    p.applyForces = 1
    p.dist00 = 1
    p.cp2 = kw.get("cp2", abi.CP2_FRICT)
    p.poisson = kw.get("poisson", 0.2)
    p.en = kw.get("en", float("nan"))
    p.law = kw.get("law", abi.LAW_IDEALELPL)
    p.noSlip = kw.get("noSlip", 0)
    p.noBreak = kw.get("noBreak", 0)
    p.noFrict = kw.get("noFrict", 0)
    p.iniEqlb = 0
    p.relRollStiff = kw.get("relRollStiff", 0.0)
    p.relTwistStiff = kw.get("relTwistStiff", 0.0)
    p.rollTanPhi = kw.get("rollTanPhi", 0.0)
    p.noAttraction = kw.get("noAttraction", 1)
    p.nMaterials = len(materials)
    p.materials = materials
    p.ellSolver = kw.get("ellSolver", abi.ELL_BRENT)
    p.brentBits = kw.get("brentBits", 32)
    p.newtonTol = kw.get("newtonTol", 1e-10)
    p.warmStart = kw.get("warmStart", abi.WARM_COLD)
    p.fallbackIters = kw.get("fallbackIters", 4)
    p.arith = kw.get("arith", abi.ARITH_EXACT)
    return p


def ellipsoid_mass_inertia(semi_axes, density):
    """Ellipsoid::lumpMassInertia (Ellipsoid.cpp:37-44): m = (4/3) pi abc rho,
    I = (1/5) m (b^2+c^2, c^2+a^2, a^2+b^2), same operation order."""
    s = np.asarray(semi_axes, np.float64).reshape(-1, 3)
    rho = np.asarray(density, np.float64)
    a, b, c = s[:, 0], s[:, 1], s[:, 2]
    m = ((4 / 3.0) * math.pi) * ((a * b) * c) * rho
    f = (1 / 5.0) * m
    inertia = np.stack([0.0 + f * (b * b + c * c), 0.0 + f * (c * c + a * a), 0.0 + f * (a * a + b * b)], axis=1)
    return m, inertia


def sphere_mass_inertia(radius, density):
    """Sphere::lumpMassInertia: m = (4/3) pi r^3 rho, I = (2/5) m r^2 (elementwise, same op order)."""
    r = np.asarray(radius, np.float64)
    rho = np.asarray(density, np.float64)
    m = ((4 / 3.0) * math.pi) * (r * r * r) * rho
    inertia = 0.0 + ((2.0 / 5.0) * m) * (r * r)
    return m, inertia


def assemble(centers, radii, sphere_mat, walls, mats_py, vel=None):
    """ParticleArrays with walls first (ids 0..nw-1), then spheres.

    walls: list of (axis, sense, position, material index)."""
    nw = len(walls)
    ns = len(radii)
    n = nw + ns
    pa = abi.ParticleArrays(n)
    for i, (ax, sense, pos, mi) in enumerate(walls):
        pa.shape[i] = abi.SHAPE_WALL
        pa.wallAxis[i] = ax
        pa.wallSense[i] = sense
        pa.pos[i, ax] = pos
        pa.material[i] = mi
        pa.mask[i] = DEFAULT_BOUNDARY_MASK
        pa.flags[i] = abi.DOF_ALL
        pa.radius[i] = np.nan
    s = slice(nw, n)
    pa.shape[s] = abi.SHAPE_SPHERE
    pa.radius[s] = radii
    pa.pos[s] = centers
    sm = np.broadcast_to(np.asarray(sphere_mat, np.int32), (ns,))
    pa.material[s] = sm
    pa.mask[s] = DEFAULT_MOVABLE_MASK
    dens = np.array([mats_py[k].get("density", 1000.0) for k in range(len(mats_py))])[sm]
    m, inert = sphere_mass_inertia(radii, dens)
    pa.mass[s] = m
    pa.inertia[s] = inert[:, None]
    if vel is not None:
        pa.vel[s] = vel
    return pa


def box_walls(lo, hi, mat=0):
    """Six axis-aligned walls of a box, each interacting towards the inside (Wall.sense)."""
    w = []
    for ax in range(3):
        w.append((ax, 1, lo[ax], mat))
        w.append((ax, -1, hi[ax], mat))
    return w


def pwave_dt(radii, mat_idx, mats_py):
    """DemFuncs::pWaveDt (src/dem/Funcs.cpp:151-175): min r / sqrt(E/rho) over spheres."""
    E = np.array([m.get("young", 1e9) for m in mats_py])[mat_idx]
    rho = np.array([m.get("density", 1000.0) for m in mats_py])[mat_idx]
    return float(np.min(radii / (1.0 * np.sqrt(E / rho))))


def spheres10k(n=10000, seed=1):
    """10k monodisperse FrictMat spheres in a walled 0.5 x 0.5 x 1.0 m box (IdealElPl)."""
    mats_py = [dict(kind=abi.MAT_FRICT, density=3000.0, young=1e7, ktDivKn=0.2, tanPhi=0.5)]
    lo, hi = np.array([0.0, 0.0, 0.0]), np.array([0.5, 0.5, 1.0])
    centers, radii = make_cloud(lo, hi, 0.005, 0.005, n, seed)
    mats = materials_array(mats_py)
    pa = assemble(centers, radii, 0, box_walls(lo, hi), mats_py)
    dt = 0.4 * pwave_dt(radii, np.zeros(len(radii), int), mats_py)
    p = default_params(mats, dt=dt, gravity=(0, 0, -9.81), damping=0.2, verletDist=-0.05)
    return SceneSpec(p, mats, pa, "spheres10k", dict(n_spheres=len(radii), seed=seed, dt=dt))


def hertz1M(n=1_000_000, seed=2, height=1.12, prefall=0.0):
    """1M polydisperse HertzMat spheres (DMT, en=.8) as a loose cloud in a 1 x 1 x 2 m walled box.

    The cloud fills z in [0, height] (height 1.12 m gives a solid fraction of about 0.3); prefall>0
    gives every sphere an initial downward velocity sqrt(2 g prefall), as after falling that far.
    For n below 1M the box and the cloud shrink by (n/1e6)^(1/3), keeping the same solid fraction
    (the "cut" of the same workload used for the CPU baseline)."""
    mats_py = [dict(kind=abi.MAT_HERTZ, density=1000.0, young=5e7, ktDivKn=0.2, tanPhi=0.3, surfEnergy=0.01),
               dict(kind=abi.MAT_HERTZ, density=1000.0, young=5e7, ktDivKn=0.2, tanPhi=0.6, surfEnergy=0.01)]
    sc = (n / 1e6) ** (1.0 / 3.0)
    lo, hi = np.array([0.0, 0.0, 0.0]), np.array([1.0, 1.0, 2.0]) * sc
    centers, radii = make_cloud(lo, np.array([1.0, 1.0, height]) * sc, 0.002, 0.006, n, seed, max_attempts=400)
    k = len(radii)
    mat_idx = (np.arange(k) % 2).astype(np.int32)
    mats = materials_array(mats_py)
    vel = None
    if prefall > 0:
        vel = np.zeros((k, 3)); vel[:, 2] = -math.sqrt(2 * 9.81 * prefall)
    pa = assemble(centers, radii, mat_idx, box_walls(lo, hi), mats_py, vel=vel)
    dt = 0.3 * pwave_dt(radii, mat_idx, mats_py)
    p = default_params(mats, dt=dt, gravity=(0, 0, -9.81), damping=0.0, verletDist=0.1 * 0.002,
                       cp2=abi.CP2_HERTZ, law=abi.LAW_HERTZ_DMT, en=0.8)
    return SceneSpec(p, mats, pa, "hertz1M" if n == 1_000_000 else f"hertz{n}", dict(n_spheres=k, seed=seed, dt=dt, height=height * sc,
                                                                                     box=hi.tolist()))


def random_cloud(n, seed, box=(0.1, 0.1, 0.1), rmin=0.004, rmax=0.006, law="frict", walls=True, vel_scale=0.5,
                 angvel_scale=5.0, gravity=(0, 0, -9.81), damping=0.2, dense=1.0, **kw):
    """Small randomised test scene: a sphere cloud squeezed by `dense` (<1 creates overlaps) with random
    velocities, optional box walls, FrictMat/IdealElPl or HertzMat/DMT."""
    rng = np.random.default_rng(seed)
    lo, hi = np.zeros(3), np.asarray(box, np.float64)
    centers, radii = make_cloud(lo, hi, rmin, rmax, n, seed)
    if dense != 1.0:
        c = hi / 2
        centers = c + (centers - c) * dense
    k = len(radii)
    vel = rng.normal(0, vel_scale, (k, 3))
    if law == "frict":
        mats_py = [dict(kind=abi.MAT_FRICT, density=2500.0, young=1e7, ktDivKn=0.2, tanPhi=0.5),
                   dict(kind=abi.MAT_FRICT, density=2000.0, young=3e7, ktDivKn=0.3, tanPhi=0.3)]
        extra = dict(cp2=abi.CP2_FRICT, law=abi.LAW_IDEALELPL)
    else:
        mats_py = [dict(kind=abi.MAT_HERTZ, density=1000.0, young=5e7, ktDivKn=0.2, tanPhi=0.3, surfEnergy=0.01),
                   dict(kind=abi.MAT_HERTZ, density=1200.0, young=8e7, ktDivKn=0.2, tanPhi=0.6, surfEnergy=0.02)]
        extra = dict(cp2=abi.CP2_HERTZ, law=abi.LAW_HERTZ_DMT, en=0.8)
    extra.update(kw)
    mat_idx = rng.integers(0, 2, k).astype(np.int32)
    mats = materials_array(mats_py)
    pa = assemble(centers, radii, mat_idx, box_walls(lo, hi) if walls else [], mats_py, vel=vel)
    nw = 6 if walls else 0
    pa.angVel[nw:] = rng.normal(0, angvel_scale, (k, 3))
    dt = 0.3 * pwave_dt(radii, mat_idx, mats_py)
    p = default_params(mats, dt=dt, gravity=gravity, damping=damping, **extra)
    # initial forces as Woo has them before the first step: m*g (ForceResetter / Leapfrog reset)
    g = np.asarray(gravity, np.float64)
    pa.force[nw:] = pa.mass[nw:, None] * g[None, :]
    return SceneSpec(p, mats, pa, f"cloud{n}", dict(seed=seed, dt=dt))


def periodic_cloud(n, seed, size=(0.1, 0.1, 0.1), rmin=0.004, rmax=0.006, law="frict", shear=0.2, rate=2.0,
                   vel_scale=0.5, angvel_scale=5.0, damping=0.0, dense=0.9, tuck=0.3, **kw):
    """Sphere cloud filling a periodic cell (Scene.isPeriodic, homoDeform gradV2).  The cloud is packed in
    the box [0, size), then positions and box are squeezed by `dense` (<1 creates overlaps) and the cell
    is a further `tuck` x rmin shorter on each axis, so spheres at opposite faces overlap through the
    boundary from the start.  hSize has an xz shear of `shear` x the z size and nextGradV a simple shear
    `rate` (1/s) of x along z.  No gravity, as usual for a cell."""
    rng = np.random.default_rng(seed)
    lo, hi = np.zeros(3), np.asarray(size, np.float64)
    centers, radii = make_cloud(lo, hi, rmin, rmax, n, seed)
    centers = centers * dense
    k = len(radii)
    L = hi * dense - tuck * rmin
    hSize = np.diag(L)
    hSize[0, 2] = shear * L[2]
    nextGradV = np.zeros((3, 3))
    nextGradV[0, 2] = rate
    if law == "frict":
        mats_py = [dict(kind=abi.MAT_FRICT, density=2500.0, young=1e7, ktDivKn=0.2, tanPhi=0.5),
                   dict(kind=abi.MAT_FRICT, density=2000.0, young=3e7, ktDivKn=0.3, tanPhi=0.3)]
        extra = dict(cp2=abi.CP2_FRICT, law=abi.LAW_IDEALELPL)
    else:
        mats_py = [dict(kind=abi.MAT_HERTZ, density=1000.0, young=5e7, ktDivKn=0.2, tanPhi=0.3, surfEnergy=0.01),
                   dict(kind=abi.MAT_HERTZ, density=1200.0, young=8e7, ktDivKn=0.2, tanPhi=0.6, surfEnergy=0.02)]
        extra = dict(cp2=abi.CP2_HERTZ, law=abi.LAW_HERTZ_DMT, en=0.8)
    extra.update(kw)
    mat_idx = rng.integers(0, 2, k).astype(np.int32)
    mats = materials_array(mats_py)
    pa = assemble(centers, radii, mat_idx, [], mats_py, vel=rng.normal(0, vel_scale, (k, 3)))
    pa.angVel[:] = rng.normal(0, angvel_scale, (k, 3))
    dt = 0.3 * pwave_dt(radii, mat_idx, mats_py)
    p = default_params(mats, dt=dt, gravity=(0, 0, 0), damping=damping, **extra)
    cell = dict(hSize=hSize, trsf=np.eye(3), gradV=np.zeros((3, 3)), nextGradV=nextGradV)
    return SceneSpec(p, mats, pa, f"peri{n}", dict(seed=seed, dt=dt), cell=cell)


def capsule_mass_inertia(radius, shaft, density):
    """Capsule::lumpMassInertia (src/dem/Capsule.cpp:44-57): mass and the principal inertia (Ix along the
    axis, Iy = Iz) of a cylinder of length shaft with hemispherical caps, in the node's frame."""
    r = np.asarray(radius, np.float64)
    s = np.asarray(shaft, np.float64)
    rho = np.asarray(density, np.float64)
    r2, r3 = r * r, r * r * r
    mCaps = (4 / 3.0) * math.pi * r3 * rho
    mShaft = math.pi * r2 * s * rho
    distCap = .5 * s + (3 / 8.0) * r
    Ix = 2 * mCaps * r2 / 5.0 + .5 * mShaft * r2
    Iy = (83 / 320.0) * mCaps * r2 + mCaps * (distCap * distCap) + (1 / 12.0) * mShaft * (3 * r2 + s * s)
    m = mCaps + mShaft
    return m, np.stack([Ix, Iy, Iy], axis=-1)


def add_capsules(pa, centers, radii, shafts, oris, mat, mats_py, vel=None, mask=None):
    """ParticleArrays with capsules appended after the particles of pa (woo.utils.capsule, py/utils.py:213-221):
    DemField.defaultMovableMask, mass and inertia from Capsule::lumpMassInertia."""
    centers = np.asarray(centers, np.float64).reshape(-1, 3)
    n0, nc = pa.n, len(centers)
    out = abi.ParticleArrays(n0 + nc)
    for k, v in pa.__dict__.items():
        if isinstance(v, np.ndarray):
            getattr(out, k)[:n0] = v
    c = slice(n0, n0 + nc)
    out.shape[c] = abi.SHAPE_CAPSULE
    out.pos[c] = centers
    out.radius[c] = radii
    out.shaft[c] = shafts
    out.ori[c] = oris
    cm = np.broadcast_to(np.asarray(mat, np.int32), (nc,))
    out.material[c] = cm
    out.mask[c] = DEFAULT_MOVABLE_MASK if mask is None else mask
    dens = np.array([mats_py[k].get("density", 1000.0) for k in range(len(mats_py))])[cm]
    m, inert = capsule_mass_inertia(np.broadcast_to(radii, (nc,)), np.broadcast_to(shafts, (nc,)), dens)
    out.mass[c] = m
    out.inertia[c] = inert
    if vel is not None:
        out.vel[c] = vel
    return out


def capsule_cloud(n_caps, n_spheres, seed, box=(0.12, 0.12, 0.12), rmin=0.003, rmax=0.005, smin=0.0, smax=0.012,
                  dense=0.85, vel_scale=0.3, gravity=(0, 0, -9.81), damping=0.2, walls=True, **kw):
    """Capsules (radius ~ U[rmin, rmax], shaft ~ U[smin, smax], random orientations) and spheres in a walled
    box, FrictMat + IdealElPl: sphere-capsule, capsule-capsule and wall-capsule contacts.  Positions come
    from a sphere packing of the capsules' bounding radii, squeezed by `dense` (<1 creates overlaps)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.zeros(3), np.asarray(box, np.float64)
    rc = rng.uniform(rmin, rmax, n_caps)
    sc = rng.uniform(smin, smax, n_caps)
    rs = rng.uniform(rmin, rmax, n_spheres)
    rin = np.concatenate([rc + .5 * sc, rs])
    centers, radii = make_cloud_radii(lo, hi, rin, seed)
    if dense != 1.0:
        mid = hi / 2
        centers = mid + (centers - mid) * dense
    # the packer returns the radii it placed (reordered, some dropped): find each one's source
    where = {}
    for j, v in enumerate(rin):
        where.setdefault(float(v), []).append(j)
    src = np.array([where[float(v)].pop(0) for v in radii], int)
    isCap = src < n_caps
    capIdx = src[isCap]
    mats_py = [dict(kind=abi.MAT_FRICT, density=2500.0, young=1e7, ktDivKn=0.2, tanPhi=0.5),
               dict(kind=abi.MAT_FRICT, density=2000.0, young=3e7, ktDivKn=0.3, tanPhi=0.3)]
    mats = materials_array(mats_py)
    sph = ~isCap
    ns = int(sph.sum())
    mat_s = rng.integers(0, 2, ns).astype(np.int32)
    pa = assemble(centers[sph], radii[sph], mat_s, box_walls(lo, hi) if walls else [], mats_py,
                  vel=rng.normal(0, vel_scale, (ns, 3)))
    ci = capIdx
    ncap = len(ci)
    pa = add_capsules(pa, centers[isCap], rc[ci], sc[ci], random_quaternions(ncap, rng), rng.integers(0, 2, ncap),
                      mats_py, vel=rng.normal(0, vel_scale, (ncap, 3)))
    nw = 6 if walls else 0
    pa.angVel[nw:] = rng.normal(0, 5.0, (pa.n - nw, 3))
    g = np.asarray(gravity, np.float64)
    pa.force[nw:] = pa.mass[nw:, None] * g[None, :]
    dt = 0.3 * pwave_dt(np.concatenate([radii[sph], rc[ci]]), np.concatenate([mat_s, np.zeros(ncap, int)]), mats_py)
    p = default_params(mats, dt=dt, gravity=gravity, damping=damping, **kw)
    return SceneSpec(p, mats, pa, f"capsules{ncap}", dict(seed=seed, dt=dt, n_capsules=ncap, n_spheres=ns))


def add_facets(pa, triangles, halfThick=0.0, mat=0):
    """ParticleArrays with fixed facets appended after the particles of pa: Facet.make defaults
    (py/utils.py:315-341) -- DemField.defaultBoundaryMask, all DOFs blocked, node masses and inertia 0;
    node 0 is the particle's position and the radius slot holds halfThick."""
    tri = np.asarray(triangles, np.float64).reshape(-1, 3, 3)
    n0, nf = pa.n, len(tri)
    out = abi.ParticleArrays(n0 + nf)
    for k, v in pa.__dict__.items():
        if isinstance(v, np.ndarray):
            getattr(out, k)[:n0] = v
    f = slice(n0, n0 + nf)
    out.shape[f] = abi.SHAPE_FACET
    out.pos[f] = tri[:, 0]
    out.facetVerts[f] = tri.reshape(nf, 9)
    out.radius[f] = halfThick
    out.material[f] = mat
    out.mask[f] = DEFAULT_BOUNDARY_MASK
    out.flags[f] = abi.DOF_ALL
    out.mass[f] = 0.0
    out.inertia[f] = 0.0
    return out


def valley_facets(lo, hi, nx, ny, depth):
    """A floor over the box's x/y extent made of nx x ny rectangles split into two triangles each, folded
    into a V along x (height depth * |x - xc| / (xc - x0) above lo[2]); vertex order gives upward normals."""
    xs = np.linspace(lo[0], hi[0], nx + 1)
    ys = np.linspace(lo[1], hi[1], ny + 1)
    xc = 0.5 * (lo[0] + hi[0])
    z = lambda x: lo[2] + depth * abs(x - xc) / (xc - lo[0])
    tris = []
    for i in range(nx):
        for j in range(ny):
            a = (xs[i], ys[j], z(xs[i]))
            b = (xs[i + 1], ys[j], z(xs[i + 1]))
            c = (xs[i + 1], ys[j + 1], z(xs[i + 1]))
            d = (xs[i], ys[j + 1], z(xs[i]))
            tris.append((a, b, c))
            tris.append((a, c, d))
    return np.array(tris)


def facet_valley(n, seed, box=(0.1, 0.1, 0.1), nx=6, ny=5, depth=0.02, halfThick=0.0, law="frict", vel_scale=0.3,
                 dense=1.0, gravity=(0, 0, -9.81), damping=0.2, **kw):
    """Spheres falling into a V-shaped valley triangulated into facets (2 nx ny Facets, halfThick), with four
    side walls: exercises facet interiors, edges and vertices."""
    rng = np.random.default_rng(seed)
    lo, hi = np.zeros(3), np.asarray(box, np.float64)
    cloud_lo = lo + np.array([0, 0, depth + 0.001])
    centers, radii = make_cloud(cloud_lo, hi, 0.004, 0.006, n, seed)
    if dense != 1.0:
        c = 0.5 * (cloud_lo + hi)
        centers = c + (centers - c) * dense
    k = len(radii)
    if law == "frict":
        mats_py = [dict(kind=abi.MAT_FRICT, density=2500.0, young=1e7, ktDivKn=0.2, tanPhi=0.5),
                   dict(kind=abi.MAT_FRICT, density=2000.0, young=3e7, ktDivKn=0.3, tanPhi=0.3)]
        extra = dict(cp2=abi.CP2_FRICT, law=abi.LAW_IDEALELPL)
    else:
        mats_py = [dict(kind=abi.MAT_HERTZ, density=1000.0, young=5e7, ktDivKn=0.2, tanPhi=0.3, surfEnergy=0.01),
                   dict(kind=abi.MAT_HERTZ, density=1200.0, young=8e7, ktDivKn=0.2, tanPhi=0.6, surfEnergy=0.02)]
        extra = dict(cp2=abi.CP2_HERTZ, law=abi.LAW_HERTZ_DMT, en=0.8)
    extra.update(kw)
    mat_idx = rng.integers(0, 2, k).astype(np.int32)
    mats = materials_array(mats_py)
    walls = [w for w in box_walls(lo, hi) if w[0] != 2]
    pa = assemble(centers, radii, mat_idx, walls, mats_py, vel=rng.normal(0, vel_scale, (k, 3)))
    nw = len(walls)
    pa.angVel[nw:] = rng.normal(0, 5.0, (k, 3))
    g = np.asarray(gravity, np.float64)
    pa.force[nw:] = pa.mass[nw:, None] * g[None, :]
    pa = add_facets(pa, valley_facets(lo, hi, nx, ny, depth), halfThick=halfThick, mat=1)
    dt = 0.3 * pwave_dt(radii, mat_idx, mats_py)
    p = default_params(mats, dt=dt, gravity=gravity, damping=damping, **extra)
    return SceneSpec(p, mats, pa, f"valley{n}", dict(seed=seed, dt=dt, n_spheres=k, n_facets=2 * nx * ny))


def quat_from_axis_angle(axis, angle):
    """Quaternion(AngleAxis(angle, axis/|axis|)) as (w, x, y, z)."""
    ax = np.asarray(axis, np.float64)
    ax = ax / math.sqrt(float(ax @ ax))
    h = 0.5 * angle
    return np.array([math.cos(h), math.sin(h) * ax[0], math.sin(h) * ax[1], math.sin(h) * ax[2]])


def quat_rotate(q, v):
    """q * v for a (w, x, y, z) quaternion: v + w uv + q.vec x uv with uv = 2 q.vec x v."""
    qv = np.asarray(q[1:], np.float64)
    v = np.asarray(v, np.float64)
    uv = np.cross(qv, v)
    uv = uv + uv
    return v + q[0] * uv + np.cross(qv, uv)


def random_quaternions(n, rng):
    """Uniformly distributed unit quaternions (Shoemake 1992, 'Uniform random rotations'), (w, x, y, z)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    a, b = np.sqrt(1 - u1), np.sqrt(u1)
    q = np.stack([b * np.cos(2 * np.pi * u3), a * np.sin(2 * np.pi * u2), a * np.cos(2 * np.pi * u2),
                  b * np.sin(2 * np.pi * u3)], axis=1)
    return q / np.linalg.norm(q, axis=1)[:, None]


def assemble_ellipsoids(centers, semi_axes, oris, mat, walls, mats_py, vel=None, spheres=None):
    """ParticleArrays: walls first, then ellipsoids (Ellipsoid.semiAxes, Node.ori), then optional spheres
    given as (centers, radii, material)."""
    nw, ne = len(walls), len(semi_axes)
    ns = 0 if spheres is None else len(spheres[1])
    n = nw + ne + ns
    pa = abi.ParticleArrays(n)
    for i, (ax, sense, pos, mi) in enumerate(walls):
        pa.shape[i] = abi.SHAPE_WALL
        pa.wallAxis[i] = ax
        pa.wallSense[i] = sense
        pa.pos[i, ax] = pos
        pa.material[i] = mi
        pa.mask[i] = DEFAULT_BOUNDARY_MASK
        pa.flags[i] = abi.DOF_ALL
    e = slice(nw, nw + ne)
    pa.shape[e] = abi.SHAPE_ELLIPSOID
    pa.semiAxes[e] = semi_axes
    pa.pos[e] = centers
    pa.ori[e] = oris
    em = np.broadcast_to(np.asarray(mat, np.int32), (ne,))
    pa.material[e] = em
    pa.mask[e] = DEFAULT_MOVABLE_MASK
    dens = np.array([mats_py[k].get("density", 1000.0) for k in range(len(mats_py))])[em]
    m, inert = ellipsoid_mass_inertia(semi_axes, dens)
    pa.mass[e] = m
    pa.inertia[e] = inert
    if vel is not None:
        pa.vel[e] = vel
    if ns:
        c, r, sm = spheres
        s = slice(nw + ne, n)
        pa.shape[s] = abi.SHAPE_SPHERE
        pa.radius[s] = r
        pa.pos[s] = c
        smi = np.broadcast_to(np.asarray(sm, np.int32), (ns,))
        pa.material[s] = smi
        pa.mask[s] = DEFAULT_MOVABLE_MASK
        d2 = np.array([mats_py[k].get("density", 1000.0) for k in range(len(mats_py))])[smi]
        m2, i2 = sphere_mass_inertia(r, d2)
        pa.mass[s] = m2
        pa.inertia[s] = i2[:, None]
    return pa


def ellipsoid_cloud(n, seed, box=(0.1, 0.1, 0.1), amin=0.004, amax=0.006, ratios=(1.0, 0.7, 0.5), walls=True,
                    vel_scale=0.5, angvel_scale=5.0, gravity=(0, 0, -9.81), damping=0.2, dense=1.0, young=1e7,
                    tanPhi=0.4, density=1000.0, dt_safety=0.9, sphere_frac=0.0, **kw):
    """Ellipsoids with semi-axes a*ratios (a uniform in [amin, amax]) and uniformly random orientations,
    placed by random sequential addition of their bounding spheres (radius a) in `box`, optionally
    squeezed by `dense` (< 1 makes overlaps); FrictMat + IdealElPl; dt = dt_safety x pWaveDt.  A fraction
    `sphere_frac` of the bodies are spheres of radius a instead (sphere + ellipsoid contacts)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.zeros(3), np.asarray(box, np.float64)
    centers, a = make_cloud(lo, hi, amin, amax, n, seed)
    if dense != 1.0:
        c = hi / 2
        centers = c + (centers - c) * dense
    sph = rng.random(len(a)) < sphere_frac
    ce, ae = centers[~sph], a[~sph]
    k = len(ae)
    semi = ae[:, None] * np.asarray(ratios, np.float64)[None, :]
    oris = random_quaternions(k, rng)
    mats_py = [dict(kind=abi.MAT_FRICT, density=density, young=young, ktDivKn=0.2, tanPhi=tanPhi)]
    mats = materials_array(mats_py)
    spheres = (centers[sph], a[sph], 0) if sph.any() else None
    pa = assemble_ellipsoids(ce, semi, oris, 0, box_walls(lo, hi) if walls else [], mats_py,
                             vel=rng.normal(0, vel_scale, (k, 3)), spheres=spheres)
    nw = 6 if walls else 0
    nb = pa.n - nw
    pa.vel[nw:] = rng.normal(0, vel_scale, (nb, 3))
    pa.angVel[nw:] = rng.normal(0, angvel_scale, (nb, 3))
    smin = semi.min(axis=1) if k else np.array([np.inf])
    if sph.any():
        smin = np.concatenate([smin, a[sph]])
    dt = dt_safety * float(np.min(smin / np.sqrt(young / density)))
    extra = dict(cp2=abi.CP2_FRICT, law=abi.LAW_IDEALELPL)
    extra.update(kw)
    p = default_params(mats, dt=dt, gravity=gravity, damping=damping, **extra)
    g = np.asarray(gravity, np.float64)
    pa.force[nw:] = pa.mass[nw:, None] * g[None, :]
    return SceneSpec(p, mats, pa, f"ell{n}", dict(seed=seed, dt=dt))


def oedometric_scene(n, seed, young, tanPhi, rmin=0.001, rmax=0.003, density=2600.0, top_vel=0.05, dt_safety=0.9,
                     dense=1.0):
    """One oedometric compression scene (after examples/oedometric.py): spheres with r ~ U[rmin, rmax] packed
    loosely (solid fraction ~0.3) in a box of base L x L and height 2L with 5 fixed walls, the top wall
    just above the topmost sphere moving down at top_vel (all DOFs blocked); particle FrictMat(young,
    ktDivKn .2, tanPhi), walls the same material without friction; gravity -10, damping 0.4.
    Returns (centers, radii, walls, mats_py, dt) for batch assembly."""
    vol = n * (4.0 / 3.0) * math.pi * ((rmax ** 4 - rmin ** 4) / (4 * (rmax - rmin))) / 0.3
    L = (vol / 2.0) ** (1.0 / 3.0)
    lo, hi = np.zeros(3), np.array([L, L, 2 * L])
    centers, radii = make_cloud(lo, hi, rmin, rmax, n, seed, max_attempts=400)
    if dense != 1.0:
        # squeezed towards the box centre: overlaps from the start (dense < 1)
        c = hi / 2
        centers = c + (centers - c) * dense
    ztop = float(np.max(centers[:, 2] + radii)) + 1e-4
    walls = [(0, 1, 0.0, 1), (0, -1, L, 1), (1, 1, 0.0, 1), (1, -1, L, 1), (2, 1, 0.0, 1), (2, -1, ztop, 1)]
    mats_py = [dict(kind=abi.MAT_FRICT, density=density, young=young, ktDivKn=0.2, tanPhi=tanPhi),
               dict(kind=abi.MAT_FRICT, density=density, young=young, ktDivKn=0.2, tanPhi=0.0)]
    dt = dt_safety * float(np.min(radii)) / math.sqrt(young / density)
    return dict(centers=centers, radii=radii, walls=walls, mats=mats_py, dt=dt, box=hi, top_vel=top_vel)


def batch_oedometric(n_scenes, seed, nmin=500, nmax=20000, spacing=None, verletDist=1e-4, dense=1.0):
    """n_scenes independent oedometric scenes in one particle set (the 512-scene batch workload): sphere counts
    log-uniform in [nmin, nmax], tanPhi ~ U[0.1, 0.8], young log-uniform in [1e6, 1e8] Pa, per-scene
    dt = 0.9 x the scene's p-wave dt (wdem_params.materialDt).  Scene k is shifted along x by k x spacing
    so the scenes stay apart; each particle carries its scene index.  Returns the SceneSpec (info holds
    the per-scene particle ranges, counts and dt)."""
    rng = np.random.default_rng(seed)
    counts = np.exp(rng.uniform(math.log(nmin), math.log(nmax), n_scenes)).astype(int)
    tanphis = rng.uniform(0.1, 0.8, n_scenes)
    youngs = np.exp(rng.uniform(math.log(1e6), math.log(1e8), n_scenes))
    parts = [oedometric_scene(int(counts[k]), seed * 100003 + k, float(youngs[k]), float(tanphis[k]), dense=dense)
             for k in range(n_scenes)]
    if spacing is None:
        spacing = 1.25 * max(float(pt["box"][0]) for pt in parts)
    ntot = sum(6 + len(pt["radii"]) for pt in parts)
    pa = abi.ParticleArrays(ntot)
    mats_py, mat_dt, ranges = [], [], []
    q = 0
    for k, pt in enumerate(parts):
        off = np.array([k * spacing, 0.0, 0.0])
        m0 = len(mats_py)
        mats_py += pt["mats"]
        mat_dt += [pt["dt"], pt["dt"]]
        ns = len(pt["radii"])
        sub = assemble(pt["centers"] + off, pt["radii"], m0, [(ax, se, pos + off[ax], m0 + mi) for ax, se, pos, mi in pt["walls"]],
                       mats_py)
        sub.vel[5] = [0.0, 0.0, -pt["top_vel"]]   # the top wall
        for name in ("shape", "radius", "wallAxis", "wallSense", "material", "mask", "flags", "mass", "inertia", "pos",
                     "ori", "vel", "angVel", "force", "torque"):
            getattr(pa, name)[q:q + 6 + ns] = getattr(sub, name)
        pa.scene[q:q + 6 + ns] = k
        ranges.append((q, q + 6 + ns))
        q += 6 + ns
    g = np.array([0.0, 0.0, -10.0])
    mov = pa.shape == abi.SHAPE_SPHERE
    pa.force[mov] = pa.mass[mov, None] * g[None, :]
    mats = materials_array(mats_py)
    dt_arr = (C_double * len(mat_dt))(*mat_dt)
    p = default_params(mats, dt=float(min(mat_dt)), gravity=tuple(g), damping=0.4, verletDist=verletDist)
    p.materialDt = dt_arr
    spec = SceneSpec(p, mats, pa, f"batch{n_scenes}",
                     dict(seed=seed, counts=[int(c) for c in counts], ranges=ranges, dt=mat_dt[::2], spacing=spacing,
                          youngs=youngs.tolist(), tanphis=tanphis.tolist()))
    spec.keep = dt_arr
    spec.scene_parts = parts
    return spec


def copy_params(p):
    """An independent copy of an abi.Params."""
    q = abi.Params()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(p), ctypes.sizeof(p))
    return q


def settle(h, spec, tail_steps=8000, dt_factor=2.5, relax_steps=2000):
    """Settle a falling cloud on the GPU handle h (untimed preparation of a packed state), with
    non-viscous damping 0.5 throughout: gravity x 10 at dt_factor x dt while the whole cloud falls (the fall
    time of its height at the damped 5 g), `tail_steps` more at 1 g and dt_factor x dt, then `relax_steps`
    at 1 g and the scene's dt.  The scene's parameters are restored afterwards (Scene.step kept).
    Returns the number of steps run."""
    p = copy_params(spec.params)
    dt = spec.params.dt
    height = spec.info.get("height", 1.0)
    g = abs(spec.params.gravity[2])
    fall = int(math.sqrt(2 * height / (5 * g)) / (dt_factor * dt))
    total = 0
    for mult, steps, f in ((10.0, fall, dt_factor), (1.0, tail_steps, dt_factor), (1.0, relax_steps, 1.0)):
        if steps <= 0:
            continue
        p.gravity[2] = spec.params.gravity[2] * mult
        p.damping = 0.5
        p.dt = dt * f
        p.step = h.status().step
        h.set_params(p)
        h.step(steps)
        total += steps
    q = copy_params(spec.params)
    q.step = h.status().step
    h.set_params(q)
    return total


def single_from_batch(spec, k):
    """Scene k of a batch as its own SceneSpec (its particles, its two materials, its dt), for checks."""
    a, b = spec.info["ranges"][k]
    n = b - a
    pa = abi.ParticleArrays(n)
    for name in ("shape", "radius", "wallAxis", "wallSense", "material", "mask", "flags", "mass", "inertia", "pos", "ori",
                 "vel", "angVel", "force", "torque"):
        getattr(pa, name)[:] = getattr(spec.particles, name)[a:b]
    m0 = int(pa.material.min())
    pa.material[:] -= m0
    mats_src = spec.materials
    mats_py = []
    for mi in (m0, m0 + 1):
        m = mats_src[mi]
        mats_py.append(dict(kind=m.kind, density=m.density, young=m.young, ktDivKn=m.ktDivKn, tanPhi=m.tanPhi,
                            surfEnergy=m.surfEnergy, alpha=m.alpha))
    mats = materials_array(mats_py)
    p = default_params(mats, dt=spec.info["dt"][k], gravity=tuple(spec.params.gravity), damping=spec.params.damping,
                       verletDist=spec.params.verletDist)
    return SceneSpec(p, mats, pa, f"scene{k}", dict(range=(a, b)))


def densify_periodic(spec, phi_target=0.62, stages=48, steps_per_stage=100, relax=600, damping=0.5, frictionless=False,
                     device=0):
    """Dense periodic packing from a loose one, on the GPU engine (the role of randomPeriPack's
    compression, py/pack.py:572): the radii grow in `stages` geometric steps to the solid fraction
    `phi_target`, each followed by `steps_per_stage` steps with non-viscous damping `damping` (and
    the scene's friction, or none) and no cell motion, then `relax` more steps in three parts.  Every
    stage and part starts from rest (velocities zeroed: the energy of the overlaps a growth step makes
    is not carried on).  The result is scaled back to the original radii (positions and cell by 1/s),
    so it is the same packing with the spec's radii in a smaller cell, and starts with the affine
    velocity field of the scene's nextGradV.  Returns a new SceneSpec with the scene's own parameters
    and cell gradients."""
    pa0 = spec.particles
    n = pa0.n
    r0 = pa0.radius.copy()
    L = float(spec.cell["hSize"][0][0])
    vs = float(np.sum((4.0 / 3.0) * math.pi * r0 ** 3))
    phi0 = vs / L ** 3
    sfin = (phi_target / phi0) ** (1.0 / 3.0)
    dens = np.array([spec.materials[int(k)].density for k in range(len(spec.materials))])[pa0.material]
    p = abi.Params()
    ctypes.memmove(ctypes.byref(p), ctypes.byref(spec.params), ctypes.sizeof(p))
    p.damping = damping
    # frictionless growth packs denser before it jams (fewer contacts at a given fraction); with the
    # scene's friction the packing jams earlier and is compressed beyond that, contact-rich
    grow_mats = (abi.Material * len(spec.materials))()
    ctypes.memmove(grow_mats, spec.materials, ctypes.sizeof(grow_mats))
    if frictionless:
        for k in range(len(grow_mats)):
            grow_mats[k].tanPhi = 0.0
    p.materials = grow_mats
    still = dict(hSize=np.diag([L, L, L]), trsf=np.eye(3), gradV=np.zeros((3, 3)), nextGradV=np.zeros((3, 3)))
    pos, ori = pa0.pos.copy(), pa0.ori.copy()
    runs = [(sfin ** (k / stages), steps_per_stage) for k in range(1, stages + 1)]
    runs += [(sfin, relax // 3)] * 3
    h = abi.Handle(n, device=device)
    try:
        for s, steps in runs:
            up = pa0.copy()
            up.pos, up.ori = pos, ori
            up.vel[:] = 0
            up.angVel[:] = 0
            up.radius = r0 * s
            m, inert = sphere_mass_inertia(up.radius, dens)
            up.mass = m
            up.inertia = np.repeat(inert[:, None], 3, axis=1)
            h.set_params(p)
            h.upload_particles(up)
            h.set_params(p)
            h.set_cell(**still)
            h.step(steps)
            st = h.download_particles(abi.ParticleArrays(n))
            pos, ori = st.pos.copy(), st.ori.copy()
    finally:
        h.close()
    out = pa0.copy()
    out.pos = pos / sfin
    out.ori = ori
    out.vel = out.pos @ np.asarray(spec.cell["nextGradV"], np.float64).T
    out.angVel[:] = 0
    Ld = L / sfin
    cell = dict(spec.cell)
    cell["hSize"] = np.diag([Ld, Ld, Ld])
    info = dict(spec.info)
    info.update(L=Ld, phi=vs / Ld ** 3, densified=dict(stages=stages, steps_per_stage=steps_per_stage, relax=relax,
                                                        damping=damping, phi_from=phi0))
    q = abi.Params()
    ctypes.memmove(ctypes.byref(q), ctypes.byref(spec.params), ctypes.sizeof(q))
    return SceneSpec(q, spec.materials, out, spec.name, info, cell=cell)


def peri_shear(n=8_000_000, seed=5, phi=0.3, rate=1.0, young=1e8, tanPhi=0.5, density=1000.0, dt_safety=0.9):
    """The periodic simple-shear workload: spheres with lognormal radii (median 1 mm, sigma 0.25, clipped to
    [0.5, 2] mm) packed without overlap (periodic random sequential addition) in a cubic periodic cell
    sized for solid fraction `phi`, simple shear nextGradV[0][2] = rate (1/s), FrictMat E `young`,
    tanPhi .5, IdealElPl, no gravity, dt = dt_safety x p-wave dt.  Random sequential addition reaches
    about 0.3; the configuration's 0.62 would need a compression run first."""
    rng = np.random.default_rng(seed)
    r = np.clip(np.exp(rng.normal(math.log(1e-3), 0.25, n)), 0.5e-3, 2e-3)
    vol = float(np.sum((4.0 / 3.0) * math.pi * r ** 3)) / phi
    L = vol ** (1.0 / 3.0)
    centers, radii = make_cloud_radii(np.zeros(3), np.array([L, L, L]), r, seed, periodic=True, max_attempts=100)
    k = len(radii)
    mats_py = [dict(kind=abi.MAT_FRICT, density=density, young=young, ktDivKn=0.2, tanPhi=tanPhi)]
    mats = materials_array(mats_py)
    pa = assemble(centers, radii, 0, [], mats_py)
    dt = dt_safety * float(np.min(radii)) / math.sqrt(young / density)
    p = default_params(mats, dt=dt, gravity=(0, 0, 0), damping=0.0)
    nextGradV = np.zeros((3, 3))
    nextGradV[0, 2] = rate
    cell = dict(hSize=np.diag([L, L, L]), trsf=np.eye(3), gradV=np.zeros((3, 3)), nextGradV=nextGradV)
    return SceneSpec(p, mats, pa, f"peri{n}", dict(seed=seed, dt=dt, L=L, phi_target=phi,
                                                   phi=float(np.sum((4 / 3) * math.pi * radii ** 3)) / L ** 3), cell=cell)
