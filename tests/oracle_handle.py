"""A stand-in for woo_gb300.abi.Handle that forwards the engine's handle calls to the oracle.

Test infrastructure: with it, the host-side layers (Scene, DemField, GpuDemEngine's bookkeeping, the
outlets) run unchanged on the CPU, and a GPU scene can be compared with the same script run on the
oracle.  Only the calls GpuDemEngine makes are provided.
"""
import ctypes as C
from types import SimpleNamespace

import numpy as np

from oracle import bridge
from woo_gb300 import abi, scenes


class OracleHandle:
    def __init__(self, max_particles, device=0):
        self.o = None
        self.params = None
        self.time_sum = 0.0
        self.max_particles = max_particles

    def _check(self, rc):
        self.o.check(rc)

    def keep_geom(self, on):
        pass

    def close(self):
        self.o = None

    def set_params(self, params):
        self.params = params
        if self.o is not None:
            self._check(self.o.lib.orc_set_params(self.o.h, C.byref(params)))

    def upload_particles(self, pa):
        if pa.n > self.max_particles:
            raise abi.WdemError(-1, "too many particles")
        self._pa = pa.copy()
        if self.o is None:
            self.o = bridge.Oracle(self.params, pa)
            return
        s = pa.struct()
        self._check(self.o.lib.orc_upload_particles(self.o.h, C.byref(s)))

    def upload_contacts(self, ca):
        s = ca.struct()
        self._check(self.o.lib.orc_upload_contacts(self.o.h, C.byref(s)))

    def set_cell(self, hSize, trsf=None, gradV=None, nextGradV=None):
        self.o.set_cell(hSize, trsf, gradV, nextGradV)

    def cell(self):
        return self.o.cell()

    def step(self, n=1):
        import time
        t0 = time.perf_counter()
        for _ in range(int(n)):
            self.time_sum += self.o.dt()
            self.o.step(1)
        self._last = (time.perf_counter() - t0) * 1e3, int(n)

    def set_timing(self, on):
        self.timing = bool(on)

    def kernel_times(self):
        """The oracle's wall time of the last step call, booked as the contact phase."""
        ms, n = getattr(self, "_last", (0.0, 0))
        return {"leapfrog": (0.0, n), "collider": (0.0, 0), "contacts": (ms, n)}

    def status(self):
        return SimpleNamespace(code=0, timeSum=self.time_sum, dt=self.o.dt(), dynDtCrit=self.o.dyndt_crit())

    def download_particles(self, pa):
        s = pa.struct()
        self.o.lib.orc_download_particles(self.o.h, C.byref(s))
        return pa

    def download_contacts(self):
        return self.o.contacts()

    def contact_count(self):
        return self.o.lib.orc_contact_count(self.o.h)

    def energy(self):
        return self.o.energy()

    # removal and insertion between steps, restated on the host: download, edit, upload (the semantics of
    # wdem_remove_particles / wdem_add_particles: removed slots inert and parked, their contacts gone, the
    # forces of the step just run kept for the next integration)
    def _state(self):
        pa = self._pa.copy()
        self.download_particles(pa)
        return pa

    def _reupload(self, pa, con):
        # the oracle takes Scene.step from the parameters: keep the current one
        q = scenes.copy_params(self.params)
        q.step = self.o.lib.orc_step_count(self.o.h)
        self.upload_particles(pa)
        self.set_params(q)
        self.upload_contacts(con)

    def remove_particles(self, ids, park=None):
        pa = self._state()
        con = self.download_contacts().without_particles(ids)
        ids = list(ids)
        pa.mask[ids] = 0
        pa.flags[ids] |= 63
        pa.vel[ids] = 0
        pa.angVel[ids] = 0
        if park is not None:
            pa.pos[ids] = park
        self._reupload(pa, con)

    def add_particles(self, particles, ids):
        pa = self._state()
        con = self.download_contacts()
        n = max(pa.n, max(ids) + 1)
        if n > pa.n:
            grown = abi.ParticleArrays(n)
            for k, v in pa.__dict__.items():
                if isinstance(v, np.ndarray):
                    getattr(grown, k)[:pa.n] = v
            pa = grown
        for k, v in particles.__dict__.items():
            if isinstance(v, np.ndarray):
                getattr(pa, k)[list(ids)] = v
        self._reupload(pa, con)


def run_on_oracle(monkeypatch, scene, n):
    """scene.run(n) with the engine's handle created on the oracle (on the first run)."""
    with monkeypatch.context() as m:
        m.setattr(abi, "Handle", OracleHandle)
        scene.run(n)
