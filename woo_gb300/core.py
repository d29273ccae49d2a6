"""Woo's Scene (woo.core.Scene, src/core/Scene.hpp / Scene.cpp) for the DEM hot path.

Scene.run/one follow Scene::doOneStep (src/core/Scene.cpp:366-467): when dt is NaN it becomes
dtSafety x min(critDt of engines and fields); the engines run in order; step and time advance.
An engine list holding Woo's [Leapfrog, InsertionSortCollider, ContactLoop] trio is run by one
GpuDemEngine built from their attributes (the drop-in replacement); any other engine is rejected.
"""
import math

from . import dem


class Labels:
    def __init__(self):
        self._d = {}

    def __getattr__(self, k):
        try:
            return self.__dict__["_d"][k]
        except KeyError:
            raise AttributeError(k)

    def _set(self, k, v):
        if k:
            self._d[k] = v


class Scene:
    """Scene (src/core/Scene.hpp:191-205 attributes dt, dtSafety, step, time, trackEnergy)."""

    def __init__(self, fields=None, engines=None, dt=float("nan"), dtSafety=0.9, trackEnergy=False):
        self.fields = list(fields or [])
        self._engines = []
        self.dt = float(dt)
        self.dtSafety = float(dtSafety)
        self.step = 0
        self.time = 0.0
        self.trackEnergy = bool(trackEnergy)
        self.lab = Labels()
        self._gpu = None
        self.engines = list(engines or [])
        for f in self.fields:
            f.scene = self

    @property
    def dem(self):
        for f in self.fields:
            if isinstance(f, dem.DemField):
                return f
        raise AttributeError("Scene has no DemField")

    @property
    def engines(self):
        return self._engines

    @engines.setter
    def engines(self, ee):
        self._engines = list(ee)
        self._gpu = None
        self.lab = Labels()
        for e in self._engines:
            self.lab._set(getattr(e, "label", ""), e)
            for lst in ("geoFunctors", "phyFunctors", "lawFunctors", "boundFunctors"):
                for f in getattr(e, lst, []):
                    self.lab._set(getattr(f, "label", ""), f)

    def _engine(self):
        if self._gpu is not None:
            return self._gpu
        ee = self._engines
        gpu = [e for e in ee if isinstance(e, dem.GpuDemEngine)]
        trio = (dem.Leapfrog, dem.InsertionSortCollider, dem.ContactLoop)
        others = [e for e in ee if not isinstance(e, (dem.GpuDemEngine,) + trio)]
        if others:
            names = ", ".join(type(e).__name__ for e in others)
            raise RuntimeError(f"engines not run by the GPU engine: {names} (DynDt: pass dynDtPeriod=0)")
        if gpu:
            self._gpu = gpu[0]
        elif all(any(isinstance(e, t) for e in ee) for t in trio):
            self._gpu = dem.GpuDemEngine.fromEngines(ee)
        else:
            raise RuntimeError("Scene.engines must hold GpuDemEngine or Leapfrog + InsertionSortCollider + ContactLoop")
        return self._gpu

    def critDt(self):
        dt = math.inf
        for e in self._engines:
            dt = min(dt, e.critDt())
        for f in self.fields:
            if hasattr(f, "critDt"):
                dt = min(dt, f.critDt())
        return dt

    def _prepare_dt(self):
        if math.isnan(self.dt) or math.isinf(self.dt) or self.dt < 0:
            dt = self.critDt()
            if math.isinf(dt):
                raise RuntimeError("Failed to obtain meaningful dt from engines and fields automatically.")
            self.dt = self.dtSafety * dt

    def run(self, nSteps=1, wait=True):
        """Run nSteps steps (the GPU runs them back to back; wait is accepted for compatibility)."""
        if nSteps <= 0:
            return
        self._prepare_dt()
        eng = self._engine()
        eng.run(self, int(nSteps))
        self.step += int(nSteps)
        self.time += self.dt * int(nSteps)

    def one(self):
        self.run(1)

    def wait(self):
        return

    @property
    def energy(self):
        """EnergyTracker (src/core/EnergyTracker.hpp): the tracked energies by name.  Slots that were
        never touched (zero) are absent, as Woo does not create them (ZeroDontCreate)."""
        if not self.trackEnergy:
            return EnergyTracker({})
        eng = self._engine()
        if eng._h is None:
            return EnergyTracker({})
        return EnergyTracker({k: v for k, v in eng._h.energy().items() if v != 0.0})


class EnergyTracker(dict):
    def total(self):
        return sum(self.values())
