"""ctypes bridge to the CPU oracle (oracle/woo_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's CPU-baseline
leg, to compare the GPU engine's results with.  It reuses the wdem.h struct layouts of woo_gb300.abi so that
both sides receive byte-identical inputs.
"""
import ctypes as C
import os

import numpy as np

from woo_gb300 import abi
from oracle import build as _build

_lib = {}


def load(variant="liborc.so"):
    if variant in _lib:
        return _lib[variant]
    libs = _build.build()
    lib = C.CDLL(libs[variant])
    h = C.c_void_p
    sig = {
        "orc_create": ([], h),
        "orc_destroy": ([h], None),
        "orc_last_error": ([h], C.c_char_p),
        "orc_set_params": ([h, C.POINTER(abi.Params)], C.c_int),
        "orc_set_mode": ([h, C.c_int, C.c_int, C.c_int], C.c_int),
        "orc_set_parallel": ([h, C.c_int], C.c_int),
        "orc_set_det_parallel": ([h, C.c_int], C.c_int),
        "orc_threads": ([], C.c_int),
        "orc_upload_particles": ([h, C.POINTER(abi.Particles)], C.c_int),
        "orc_upload_contacts": ([h, C.POINTER(abi.Contacts)], C.c_int),
        "orc_step": ([h, C.c_int], C.c_int),
        "orc_step_timed": ([h, C.c_int], C.c_double),
        "orc_download_particles": ([h, C.POINTER(abi.Particles)], C.c_int),
        "orc_contact_count": ([h], C.c_long),
        "orc_download_contacts": ([h, C.POINTER(abi.Contacts)], C.c_int),
        "orc_crit_dt": ([h], C.c_double),
        "orc_get_dt": ([h], C.c_double),
        "orc_dyndt_crit": ([h], C.c_double),
        "orc_get_energy": ([h, C.POINTER(C.c_double), C.c_int], C.c_int),
        "orc_reset_energy": ([h], C.c_int),
        "orc_nfullruns": ([h], C.c_long),
        "orc_ell_stats": ([h, C.POINTER(C.c_long), C.POINTER(C.c_long)], C.c_int),
        "orc_verlet_dist": ([h], C.c_double),
        "orc_step_count": ([h], C.c_long),
        "orc_set_update_phys": ([h, C.c_int], C.c_int),
        "orc_set_young": ([h, C.c_int, C.c_double], C.c_int),
        "orc_set_cell": ([h, C.c_int, abi.D], C.c_int),
        "orc_get_cell": ([h, abi.D], C.c_int),
        "orc_stress": ([h, abi.D], C.c_int),
        "orc_collide_boxes": ([C.c_int, abi.D, abi.D, abi.U32, C.c_uint32, C.c_int, abi.I32, C.c_long], C.c_long),
        "orc_collide_frames": ([C.c_int, C.c_int, abi.D, abi.D, abi.U32, C.c_uint32, abi.I32, C.c_long], C.c_long),
        "orc_make_cloud": ([abi.D, abi.D, C.c_double, C.c_double, C.c_int64, C.c_uint64, C.c_int32, abi.D, abi.D],
                           C.c_int64),
        "orc_make_cloud_radii": ([abi.D, abi.D, C.c_int32, C.c_int64, abi.D, C.c_uint64, C.c_int32, abi.D, abi.D],
                                 C.c_int64),
        "orc_sort_passes": ([h], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    _lib[variant] = lib
    return lib


class Oracle:
    """One CPU restatement of Woo's DEM scene (Leapfrog, InsertionSortCollider, ContactLoop)."""

    def __init__(self, params, particles, contacts=None, canonical=True, sort_axis=0, variant="liborc.so", cell=None,
                 threads=False):
        """threads=True: the OpenMP build with loops that give the serial results bit for bit (canonical
        runs only), for the long parity runs."""
        if threads:
            variant = "liborc_omp.so"
        self.lib = load(variant)
        self.h = self.lib.orc_create()
        self._params = params
        self.lib.orc_set_mode(self.h, 1 if canonical else 0, 1 if canonical else 0, sort_axis)
        self.check(self.lib.orc_set_params(self.h, C.byref(params)))
        if cell is not None:
            self.set_cell(**cell)
        s = particles.struct()
        self.check(self.lib.orc_upload_particles(self.h, C.byref(s)))
        self.check(self.lib.orc_set_params(self.h, C.byref(params)))
        if contacts is not None:
            cs = contacts.struct()
            self.check(self.lib.orc_upload_contacts(self.h, C.byref(cs)))
        self.n = particles.n
        if threads:
            if not canonical:
                raise ValueError("threads=True reproduces the canonical serial oracle only")
            self.check(self.lib.orc_set_det_parallel(self.h, 1))

    def check(self, rc):
        if rc != 0:
            raise RuntimeError("oracle: " + (self.lib.orc_last_error(self.h) or b"").decode())

    def __del__(self):
        try:
            if self.h:
                self.lib.orc_destroy(self.h)
        except Exception:
            pass

    def set_parallel(self, on=True):
        """OpenMP contact/node loops (liborc_omp.so only): the reference's parallel scheme, for timing."""
        if self.lib.orc_set_parallel(self.h, 1 if on else 0) != 0:
            raise RuntimeError("this oracle build has no OpenMP")

    def threads(self):
        return self.lib.orc_threads()

    def sort_passes(self):
        """Passes of the last parallel insertion sort (OpenMP build)."""
        return self.lib.orc_sort_passes(self.h)

    def step(self, n=1):
        self.check(self.lib.orc_step(self.h, int(n)))

    def step_timed(self, n):
        t = self.lib.orc_step_timed(self.h, int(n))
        if t < 0:
            self.check(-1)
        return t

    def particles(self):
        pa = abi.ParticleArrays(self.n)
        s = pa.struct()
        self.lib.orc_download_particles(self.h, C.byref(s))
        return pa

    def contacts(self):
        ca = abi.ContactArrays(self.lib.orc_contact_count(self.h))
        s = ca.struct()
        self.lib.orc_download_contacts(self.h, C.byref(s))
        return ca

    def crit_dt(self):
        return self.lib.orc_crit_dt(self.h)

    def set_cell(self, hSize, trsf=None, gradV=None, nextGradV=None):
        """Periodic cell: 3x3 hSize (columns = base vectors), trsf, gradV, nextGradV."""
        m = np.zeros(36)
        m[0:9] = np.asarray(hSize, float).reshape(9)
        m[9:18] = np.asarray(trsf if trsf is not None else np.eye(3), float).reshape(9)
        m[18:27] = np.asarray(gradV if gradV is not None else np.zeros((3, 3)), float).reshape(9)
        m[27:36] = np.asarray(nextGradV if nextGradV is not None else np.zeros((3, 3)), float).reshape(9)
        self.lib.orc_set_cell(self.h, 1, abi.ptr(m, C.c_double))

    def cell(self):
        m = np.zeros(45)
        self.lib.orc_get_cell(self.h, abi.ptr(m, C.c_double))
        return dict(hSize=m[0:9].reshape(3, 3), trsf=m[9:18].reshape(3, 3), gradV=m[18:27].reshape(3, 3),
                    nextGradV=m[27:36].reshape(3, 3), pprevHsize=m[36:45].reshape(3, 3))

    def stress(self):
        m = np.zeros(9)
        self.lib.orc_stress(self.h, abi.ptr(m, C.c_double))
        return m.reshape(3, 3)

    def energy(self):
        e = (C.c_double * 8)()
        self.lib.orc_get_energy(self.h, e, 8)
        return dict(zip(abi.ENERGY_NAMES, list(e)))

    def reset_energy(self):
        self.lib.orc_reset_energy(self.h)

    def dt(self):
        return self.lib.orc_get_dt(self.h)

    def dyndt_crit(self):
        return self.lib.orc_dyndt_crit(self.h)

    def n_full_runs(self):
        return self.lib.orc_nfullruns(self.h)

    def ell_stats(self):
        """(solves, contact-function evaluations) of the ellipsoid functors so far."""
        a, b = C.c_long(), C.c_long()
        self.lib.orc_ell_stats(self.h, C.byref(a), C.byref(b))
        return a.value, b.value

    def verlet_dist(self):
        return self.lib.orc_verlet_dist(self.h)

    def set_update_phys(self, up):
        self.lib.orc_set_update_phys(self.h, up)

    def set_young(self, mat, young):
        self.lib.orc_set_young(self.h, mat, young)


def collide_boxes(mins, maxs, mask, lone_mask, sort_axis=0):
    """InsertionSortCollider initial sort + sweep over the given boxes; returns sorted (min,max) pairs."""
    lib = load()
    mins = np.ascontiguousarray(mins, np.float64)
    maxs = np.ascontiguousarray(maxs, np.float64)
    mask = np.ascontiguousarray(mask, np.uint32)
    n = len(mins)
    cnt = lib.orc_collide_boxes(n, abi.ptr(mins, C.c_double), abi.ptr(maxs, C.c_double), abi.ptr(mask, C.c_uint32),
                                lone_mask, sort_axis, None, 0)
    pairs = np.zeros((max(cnt, 1), 2), np.int32)
    lib.orc_collide_boxes(n, abi.ptr(mins, C.c_double), abi.ptr(maxs, C.c_double), abi.ptr(mask, C.c_uint32),
                          lone_mask, sort_axis, abi.ptr(pairs, C.c_int32), cnt)
    return pairs[:cnt]


def collide_frames(mins, maxs, mask, lone_mask):
    """Insertion-sort collider run over successive box sets (frames x n x 3); pairs after the last."""
    lib = load()
    mins = np.ascontiguousarray(mins, np.float64)
    maxs = np.ascontiguousarray(maxs, np.float64)
    mask = np.ascontiguousarray(mask, np.uint32)
    nf, n = mins.shape[0], mins.shape[1]
    cnt = lib.orc_collide_frames(n, nf, abi.ptr(mins, C.c_double), abi.ptr(maxs, C.c_double),
                                 abi.ptr(mask, C.c_uint32), lone_mask, None, 0)
    pairs = np.zeros((max(cnt, 1), 2), np.int32)
    lib.orc_collide_frames(n, nf, abi.ptr(mins, C.c_double), abi.ptr(maxs, C.c_double), abi.ptr(mask, C.c_uint32),
                           lone_mask, abi.ptr(pairs, C.c_int32), cnt)
    return pairs[:cnt]


def make_cloud(lo, hi, rmin, rmax, n, seed, max_attempts=200, variant="liborc.so"):
    """The benchmark's seeded sphere cloud built by the oracle's restatement of the engine's generator
    (identical arrays to woo_gb300.abi.make_cloud); returns (centers (k,3), radii (k,))."""
    lib = load(variant)
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    centers = np.zeros((n, 3))
    radii = np.zeros(n)
    k = lib.orc_make_cloud(abi.ptr(lo, C.c_double), abi.ptr(hi, C.c_double), float(rmin), float(rmax), int(n),
                           int(seed), int(max_attempts), abi.ptr(centers, C.c_double), abi.ptr(radii, C.c_double))
    if k < 0:
        raise RuntimeError("orc_make_cloud: bad arguments")
    return centers[:k].copy(), radii[:k].copy()


def make_cloud_radii(lo, hi, radii_in, seed, periodic=False, max_attempts=200, variant="liborc.so"):
    """The oracle's restatement of woo_gb300.abi.make_cloud_radii (identical arrays)."""
    lib = load(variant)
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    rin = np.ascontiguousarray(radii_in, np.float64)
    n = len(rin)
    centers = np.zeros((n, 3))
    radii = np.zeros(n)
    k = lib.orc_make_cloud_radii(abi.ptr(lo, C.c_double), abi.ptr(hi, C.c_double), 1 if periodic else 0, n,
                                 abi.ptr(rin, C.c_double), int(seed), int(max_attempts), abi.ptr(centers, C.c_double),
                                 abi.ptr(radii, C.c_double))
    if k < 0:
        raise RuntimeError("orc_make_cloud_radii: bad arguments")
    return centers[:k].copy(), radii[:k].copy()
