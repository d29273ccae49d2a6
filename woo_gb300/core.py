"""Woo's Scene (woo.core.Scene, src/core/Scene.hpp / Scene.cpp) for the DEM hot path.

Scene.run/one follow Scene::doOneStep (src/core/Scene.cpp:366-467): when dt is NaN it becomes
dtSafety x min(critDt of engines and fields); the engines run in order; step and time advance.
An engine list holding Woo's [Leapfrog, InsertionSortCollider, ContactLoop] trio is run by one
GpuDemEngine built from their attributes (the drop-in replacement); DynDt runs inside it and
periodic host engines (outlets) between its steps; any other engine is rejected.
"""
import math

import numpy as np

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


class Cell:
    """Cell (src/core/Cell.hpp:22-187), homoDeform gradV2: hSize (columns = cell vectors), trsf, gradV,
    nextGradV (the velocity gradient applied from the next step).  Read back after every run."""

    _HOMO = ("none", "pos", "vel", "vel2", "gradV2")

    def __init__(self):
        self._hSize = np.eye(3)
        self._trsf = np.eye(3)
        self._gradV = np.zeros((3, 3))
        self._nextGradV = np.zeros((3, 3))
        self._homoDeform = "gradV2"
        self._edited = True

    @property
    def homoDeform(self):
        return self._homoDeform

    @homoDeform.setter
    def homoDeform(self, v):
        """Cell::homoDeform (Cell.hpp:135): only the default gradV2 integration is provided."""
        v = self._HOMO[v] if isinstance(v, int) else str(v)
        if v not in self._HOMO:
            raise ValueError(f"Cell.homoDeform: unknown mode {v!r}")
        if v != "gradV2":
            raise RuntimeError(f"Cell.homoDeform={v!r} is not supported (only 'gradV2')")
        self._homoDeform = v

    def _prop(name):
        def get(self):
            return getattr(self, "_" + name).copy()

        def set_(self, v):
            m = np.asarray(v, np.float64).reshape(3, 3).copy()
            if name == "hSize" and np.linalg.det(m) <= 0:
                # Cell::setHSize / integrateAndUpdate: a degenerate (or inverted) cell is an error
                raise RuntimeError("Cell.hSize: degenerate or inverted cell (det(hSize) <= 0)")
            setattr(self, "_" + name, m)
            self._edited = True
        return property(get, set_)

    hSize = _prop("hSize")
    trsf = _prop("trsf")
    gradV = _prop("gradV")
    nextGradV = _prop("nextGradV")
    del _prop

    def setBox(self, *box):
        """Cell.setBox: rectangular cell of the given size."""
        size = box[0] if len(box) == 1 else box
        self.hSize = np.diag(np.asarray(size, np.float64).reshape(3))

    @property
    def hSize0(self):
        """Reference cell: trsf^-1 · hSize."""
        return np.linalg.solve(self._trsf, self._hSize)

    @property
    def size(self):
        return np.linalg.norm(self._hSize, axis=0)

    @property
    def volume(self):
        return float(np.linalg.det(self._hSize))

    def _sync(self, d):
        self._hSize, self._trsf, self._gradV = d["hSize"], d["trsf"], d["gradV"]
        self._nextGradV = d["nextGradV"]
        self._edited = False


_TMP = {}   # scenes kept in memory by Scene.saveTmp


class Scene:
    """Scene (src/core/Scene.hpp:191-205 attributes dt, dtSafety, step, time, trackEnergy, isPeriodic, cell)."""

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
        self._host = []
        self._host_energy = {}
        self.stopAtStep = 0
        self.stopAtTime = float("nan")
        self.stopAtHook = ""
        self.periodic = False
        self.cell = Cell()
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
        self._host = []
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
        dyn = [e for e in ee if isinstance(e, dem.DynDt)]
        host = [e for e in ee if isinstance(e, dem.PeriodicEngine) and type(e).run is not dem.PeriodicEngine.run]
        others = [e for e in ee if not isinstance(e, (dem.GpuDemEngine, dem.DynDt) + trio) and e not in host]
        if others:
            names = ", ".join(type(e).__name__ for e in others)
            raise RuntimeError(f"engines not run by the GPU engine: {names}")
        if len(dyn) > 1:
            raise RuntimeError("more than one DynDt engine")
        if gpu:
            self._gpu = gpu[0]
        elif all(any(isinstance(e, t) for e in ee) for t in trio):
            self._gpu = dem.GpuDemEngine.fromEngines(ee)
        else:
            raise RuntimeError("Scene.engines must hold GpuDemEngine or Leapfrog + InsertionSortCollider + ContactLoop")
        self._gpu._dynDt = dyn[0] if dyn else None
        for e in host:
            e._check()
        self._host = host
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

    def run(self, steps=-1, wait=True, time=float("nan"), nSteps=None):
        """Scene.run(steps, wait, time) (src/core/Scene.cpp): `steps` > 0 sets stopAtStep = step + steps,
        `time` sets stopAtTime = time + `time`; the run ends at stopAtStep, or after the first step that
        brings Scene.time to stopAtTime.  The GPU engine runs synchronously, so `wait` changes nothing,
        and a run without a stop condition is an error instead of a loop without end.  steps=0 returns
        at once."""
        if nSteps is not None:
            steps = nSteps
        if steps == 0:
            return
        if steps is not None and steps > 0:
            self.stopAtStep = self.step + int(steps)
        if not math.isnan(time):
            self.stopAtTime = self.time + time
        if self.stopAtHook:
            raise RuntimeError("Scene.stopAtHook (a Python string run by Woo) is not supported")
        by_step = self.stopAtStep > self.step
        by_time = not math.isnan(self.stopAtTime) and self.time < self.stopAtTime
        if not by_step and not by_time:
            raise RuntimeError("Scene.run: nothing to run until (give steps or time, or set stopAtStep / stopAtTime "
                               "beyond the current step and time)")
        self._prepare_dt()
        while True:
            k = self.stopAtStep - self.step if by_step else None
            if by_time:
                est = int((self.stopAtTime - self.time) / self.dt) - 2
                kt = max(est, 1)
                dyn = [e for e in self._engines if isinstance(e, dem.DynDt) and e.stepPeriod > 0]
                if dyn and est > 1:
                    # a new dt takes effect after a DynDt step: keep it constant within the chunk
                    per = int(dyn[0].stepPeriod)
                    kt = min(kt, (-(-self.step // per) * per) - self.step + 1)
                k = kt if k is None else min(k, kt)
            self._run_steps(max(int(k), 1))
            if by_step and self.step >= self.stopAtStep:
                break
            if by_time and self.time >= self.stopAtTime:
                break

    def _run_steps(self, nSteps):
        """nSteps steps: the GPU runs them back to back, stopping after the contact pass of each step at
        which a host engine (an outlet, an inlet) is due; that engine then runs with step, time, dt and
        cell.gradV as Scene::doOneStep has them while its engines run (before the epilogue,
        src/core/Scene.cpp:428-432).  Without engines only step and time advance."""
        if not self._engines and self._gpu is None:
            for _ in range(int(nSteps)):
                self.step += 1
                self.time += self.dt
            return
        eng = self._engine()
        end = self.step + int(nSteps)
        while self.step < end:
            due = [e._next_step(self.step, self.time) for e in self._host]
            due = [t for t in due if t is not None and t < end]
            if not due:
                self._gpu_steps(eng, end - self.step)
                break
            t = min(due)
            if t > self.step:
                self._gpu_steps(eng, t - self.step)
            dt, gradV, time = self.dt, self.cell.gradV, self.time
            eng.run(self, 1)
            new_dt, new_gradV = self.dt, self.cell._gradV
            self.dt = dt
            self.cell._gradV = gradV
            try:
                for e in self._host:
                    if e._activate(self.step, time):
                        e.run(self)
            finally:
                self.dt = new_dt
                self.cell._gradV = new_gradV
            self.step += 1
            self._advance_time(eng)

    def _gpu_steps(self, eng, k):
        eng.run(self, int(k))
        self.step += int(k)
        self._advance_time(eng)

    def _advance_time(self, eng):
        t = getattr(eng, "_time_after", None)
        self.time = t if t is not None else self.time + eng._ran_time

    def _energy_add(self, name, value):
        """EnergyTracker::add with ZeroDontCreate|IsIncrement, for energies booked on the host."""
        if value == 0.0 and name not in self._host_energy:
            return
        self._host_energy[name] = self._host_energy.get(name, 0.0) + value

    def save(self, path):
        """Scene.save: the scene as a pickle (format of this package, not Woo's archives): particles with
        their current state, the contact container with its history, engines and host engines with
        their counters, the periodic cell, step, time, dt and the energies booked so far.  Loading
        it (Scene.load) and running continues the motion; the first step runs the collider in full.
        Not kept: DynDt's device-side schedule (it restarts with its next period) and the cell's
        previous-step size."""
        import pickle
        with open(path, "wb") as f:
            pickle.dump(self, f, protocol=pickle.HIGHEST_PROTOCOL)

    @staticmethod
    def load(path):
        import pickle
        with open(path, "rb") as f:
            S = pickle.load(f)
        if not isinstance(S, Scene):
            raise TypeError("Loaded object of type " + type(S).__name__ + " is not a Scene")
        return S

    def saveTmp(self, name="", quiet=False):
        """Scene.saveTmp: the scene kept in memory under `name` (as Scene.save writes it)."""
        import pickle
        _TMP[name] = pickle.dumps(self, protocol=pickle.HIGHEST_PROTOCOL)

    @staticmethod
    def loadTmp(name=""):
        """Scene.loadTmp: a new scene from the state saved by saveTmp under `name`."""
        import pickle
        if name not in _TMP:
            raise ValueError(f"No memory-saved scene named {name!r}")
        return pickle.loads(_TMP[name])

    def __getstate__(self):
        d = dict(self.__dict__)
        for fld in self.fields:
            if getattr(fld, "_engine", None) is not None and fld._stale:
                fld._engine._download_particles(fld)
        return d

    @property
    def running(self):
        """Scene.running: a run returns only when its steps are done, so no run is in progress between
        calls."""
        return False

    def stop(self):
        """Scene.stop: nothing runs in the background, so there is nothing to stop."""
        return None

    def paused(self):
        """Scene.paused(): a context manager; with synchronous runs it only brackets the block."""
        import contextlib
        return contextlib.nullcontext(self)

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
            return EnergyTracker(dict(self._host_energy))
        d = {k: v for k, v in eng.energy().items() if v != 0.0}
        d.update(self._host_energy)
        return EnergyTracker(d)


class EnergyTracker(dict):
    def total(self):
        return sum(self.values())
