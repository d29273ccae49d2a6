"""woo.models.ContactModelSelector (py/models.py:212-315) for the contact models the GPU engine runs.

It maps a model name to the Cp2/Law2 functors and the Leapfrog damping that DemField.minimalEngines
(model=...) puts into the engine list:
- 'linear': Cp2_FrictMat_FrictPhys + Law2_L6Geom_FrictPhys_IdealElPl (rolling with linRoll);
- 'Hertz', 'DMT', 'Schwarz': Cp2_HertzMat_HertzPhys(poisson, en=restitution) + Law2_L6Geom_HertzPhys_DMT.

The engine runs the DMT branch of that law: a 'Schwarz' scene (HertzMat with alpha != 0 and
surfEnergy != 0) is refused when the engine starts.  The other models of the reference (pellet,
concrete, ice, luding) have no GPU counterpart and are refused here.
"""
from . import dem

MODELS = ("linear", "pellet", "Hertz", "DMT", "Schwarz", "concrete", "ice", "luding")
PROVIDED = ("linear", "Hertz", "DMT", "Schwarz")
# the reference lists FrictMat for 'Hertz' and 'DMT' (py/models.py:304-309), but Cp2_HertzMat_HertzPhys
# dispatches on (HertzMat, HertzMat) only (src/dem/Hertz.hpp:54), so those scenes fail at their first
# contact there (ContactLoop.cpp:181); HertzMat is used for all three Hertzian models here
_MAT_CLASS = {"linear": dem.FrictMat, "Hertz": dem.HertzMat, "DMT": dem.HertzMat, "Schwarz": dem.HertzMat}


class ContactModelSelector(dem._Attrs):
    """name, numMat (min, max number of materials), matDesc, mats, distFactor, poisson, restitution,
    damping, linRoll, linRollParams (relRollStiff, relTwistStiff, rollTanPhi); alpha and surfEnergy
    are the reference's deprecated attributes and must stay zero."""
    _defaults = dict(name="linear", numMat=(1, 1), matDesc=(), mats=(), distFactor=1.0, poisson=0.2,
                     restitution=1.0, damping=0.2, linRoll=False, linRollParams=(1.0, 1.0, 1.0), alpha=0.0,
                     surfEnergy=0.0)

    def __init__(self, **kw):
        super().__init__(**kw)
        self.mats = list(self.mats)
        self.postLoad()

    def postLoad(self, what=None):
        """ContactModelSelector.postLoad (py/models.py:244-275): material count within numMat, material
        classes matching the model (attributes carried over), deprecated attributes refused."""
        if self.name not in MODELS:
            raise ValueError("Unknown model: " + str(self.name))
        lo, hi = self.numMat
        if len(self.mats) > hi:
            self.mats = self.mats[:hi]
        elif len(self.mats) < lo:
            self.mats += [self.getMat() for _ in range(lo - len(self.mats))]
        for i, m0 in enumerate(self.mats):
            if type(m0) is not self.getMatClass():
                m = self.getMat()
                for k in m.__dict__:
                    if hasattr(m0, k):
                        setattr(m, k, getattr(m0, k))
                self.mats[i] = m
        if self.alpha != 0. or self.surfEnergy != 0:
            raise ValueError("ContactModelSelector.alpha or ContactModelSelector.surfEnergy are non-zero. "
                             "Do not use those anymore.")

    def getFunctors(self):
        """([CPhysFunctor], [LawFunctor]) of the selected model (py/models.py:277-300)."""
        if self.name == "linear":
            law = dem.Law2_L6Geom_FrictPhys_IdealElPl()
            if self.linRoll:
                law.relRollStiff, law.relTwistStiff, law.rollTanPhi = self.linRollParams
            return [dem.Cp2_FrictMat_FrictPhys()], [law]
        if self.name in ("Hertz", "DMT", "Schwarz"):
            return [dem.Cp2_HertzMat_HertzPhys(poisson=self.poisson, en=self.restitution)], [dem.Law2_L6Geom_HertzPhys_DMT()]
        raise ValueError(f"ContactModelSelector: model {self.name!r} has no GPU counterpart "
                         f"(provided: {', '.join(PROVIDED)})")

    def getMatClass(self):
        if self.name not in _MAT_CLASS:
            if self.name in MODELS:
                raise ValueError(f"ContactModelSelector: model {self.name!r} has no GPU counterpart "
                                 f"(provided: {', '.join(PROVIDED)})")
            raise ValueError("Unknown model: " + str(self.name))
        return _MAT_CLASS[self.name]

    def getMat(self):
        return self.getMatClass()()

    def getNonviscDamping(self):
        """Leapfrog.damping for the model: `damping` for 'linear' (and 'ice'), zero for the models with
        their own damping (py/models.py:312-315)."""
        return self.damping if self.name in ("linear", "ice") else 0.
