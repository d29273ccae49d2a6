"""woo.utils slice for the DEM hot path (py/utils.py): defaultEngines / DemField.minimalEngines,
sphere/ellipsoid/facet/wall constructors, defaultMaterial."""
import math
import warnings

from . import dem
from .dem import defaultMaterial  # noqa: F401


def defaultEngines(damping=0.0, gravity=None, verletDist=-0.05, kinSplit=False, dontCollect=False, noSlip=False,
                   noBreak=False, cp2=None, law=None, model=None, collider="sap", grid=None, dynDtPeriod=100,
                   cpKw={}, lawKw={}):
    """py/utils.py:94-129: [Leapfrog(reset=True), InsertionSortCollider, ContactLoop(...)] (+ DynDt).
    dynDtPeriod=0 leaves DynDt out."""
    if gravity:
        raise ValueError("gravity MUST NOT be specified anymore, set DemField.gravity=... instead.")
    if model is not None:
        # py/utils.py:100-108: the functors and the damping come from the ContactModelSelector
        if cp2 or law:
            warnings.warn("cp2 and law args are ignored when model is provided.")
        if damping != 0.:
            warnings.warn("damping is ignored when model is provided.")
        cp2, law = model.getFunctors()
        if len(law) == 1:
            law[0].label = "contactLaw"
        if len(cp2) == 1:
            cp2[0].label = "cp2"
        damping = model.getNonviscDamping()
        if model.distFactor != 1.0:
            raise ValueError("ContactModelSelector.distFactor is not copied into the engines; set DemField.distFactor")
    else:
        cp2 = [cp2 if cp2 else dem.Cp2_FrictMat_FrictPhys()]
        law = [law if law else dem.Law2_L6Geom_FrictPhys_IdealElPl(noSlip=noSlip, noBreak=noBreak, label="contactLaw")]
    for k, v in cpKw.items():
        setattr(cp2[0], k, v)
    for k, v in lawKw.items():
        setattr(law[0], k, v)
    if collider != "sap":
        raise ValueError("only the sweep-and-prune collider ('sap') is provided")
    engines = [
        dem.Leapfrog(damping=damping, reset=True, kinSplit=kinSplit, dontCollect=dontCollect, label="leapfrog"),
        dem.InsertionSortCollider([dem.Bo1_Sphere_Aabb(), dem.Bo1_Facet_Aabb(), dem.Bo1_Wall_Aabb(), dem.Bo1_Capsule_Aabb()],
                                  label="collider", verletDist=verletDist),
        dem.ContactLoop([dem.Cg2_Sphere_Sphere_L6Geom(), dem.Cg2_Facet_Sphere_L6Geom(), dem.Cg2_Wall_Sphere_L6Geom(),
                         dem.Cg2_Wall_Capsule_L6Geom(), dem.Cg2_Capsule_Capsule_L6Geom(),
                         dem.Cg2_Sphere_Capsule_L6Geom()],
                        cp2, law, applyForces=True, label="contactLoop"),
    ]
    if dynDtPeriod > 0:
        engines.append(dem.DynDt(stepPeriod=dynDtPeriod, label="dynDt"))
    return engines


def sphere(center, radius, mat=None, fixed=False, wire=False, color=None, highlight=False,
           mask=dem.DEFAULT_MOVABLE_MASK, vel=None):
    """py/utils.py:153-199."""
    return dem.Sphere.make(center, radius, mat=mat, fixed=fixed, mask=mask, vel=vel)


def ellipsoid(center, semiAxes, ori=(1, 0, 0, 0), angVel=None, color=None, mat=None, fixed=False, wire=False,
              visible=True, mask=dem.DEFAULT_MOVABLE_MASK, **kw):
    """py/utils.py:201-211: an Ellipsoid particle (ori as (w, x, y, z)); angVel sets the node's angular
    velocity."""
    p = dem.Ellipsoid.make(center, semiAxes, ori=ori, mat=mat, fixed=fixed, mask=mask)
    if angVel is not None:
        p.angVel = angVel
    return p


def capsule(center, radius, shaft, ori=(1, 0, 0, 0), fixed=False, color=None, wire=False, mat=None,
            mask=dem.DEFAULT_MOVABLE_MASK):
    """py/utils.py:213-221: a Capsule on a new node with orientation ori (w, x, y, z)."""
    return dem.Capsule.make(center, radius, shaft, ori=ori, mat=mat, fixed=fixed, mask=mask)


def facet(vertices, fakeVel=None, halfThick=0.0, fixed=True, wire=True, color=None, highlight=False, mat=None,
          visible=True, mask=dem.DEFAULT_BOUNDARY_MASK):
    """py/utils.py:315-341: a Facet of three new nodes."""
    return dem.Facet.make(vertices, halfThick=halfThick, mat=mat, fixed=fixed, mask=mask, fakeVel=fakeVel)


def wall(position, axis, sense=0, glAB=None, fixed=True, mass=0, color=None, mat=None, visible=True,
         mask=dem.DEFAULT_BOUNDARY_MASK):
    """py/utils.py:245-267."""
    return dem.Wall.make(position, axis, sense=sense, mat=mat, fixed=fixed, mass=mass, mask=mask)


def wallBox(box, which=(1, 1, 1, 1, 1, 1), **kw):
    """py/utils.py:269-: six walls of an axis-aligned box facing inwards."""
    lo, hi = box
    out = []
    for ax in range(3):
        if which[2 * ax]:
            out.append(wall(lo[ax], ax, sense=1, **kw))
        if which[2 * ax + 1]:
            out.append(wall(hi[ax], ax, sense=-1, **kw))
    return out


def spherePWaveDt(radius, density, young):
    """py/utils.py:77-: r / sqrt(E/rho)."""
    return radius / math.sqrt(young / density)


def unbalancedEnergy(S):
    """py/utils.py:757-763: kinetic over elastic energy (NaN when either is missing or elast is 0)."""
    if not S.trackEnergy:
        raise RuntimeError("Scene.trackEnergy==False")
    e = S.energy
    if "elast" not in e or "kinetic" not in e or e["elast"] == 0:
        return float("nan")
    return e["kinetic"] / e["elast"]


def unbalancedForce(S=None, useMaxForce=False, field=None):
    """DemFuncs::unbalancedForce of the scene's DemField (see DemField.unbalancedForce)."""
    return (field if field is not None else S.dem).unbalancedForce(useMaxForce)
