"""ctypes mirror of include/wdem.h and the loader of libwdem.so.

The library is the only compute path: if it cannot be loaded, every engine call raises.  There is
no CPU fallback.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libwdem.so")

ABI_VERSION = 2

# error codes
WDEM_OK = 0
WDEM_ERR_ARG = -1
WDEM_ERR_CUDA = -2
WDEM_ERR_NAN = -3
WDEM_ERR_OVERFLOW = -4
WDEM_ERR_UNSUPPORTED = -5
WDEM_ERR_NO_PHYS = -6
WDEM_ERR_TOO_BIG = -7
WDEM_ERR_TIMEOUT = -8
WDEM_ERR_STATE = -9

SHAPE_SPHERE, SHAPE_WALL, SHAPE_ELLIPSOID, SHAPE_FACET, SHAPE_CAPSULE = 0, 1, 2, 3, 4
ELL_BRENT, ELL_NEWTON = 0, 1
WARM_INPUTS, WARM_OUTPUTS, WARM_RECORD, WARM_NPARAM = 13, 4, 17, 9476
WARM_COLD, WARM_MLP, WARM_HISTORY, WARM_HISTORY_MLP = 0, 1, 2, 3
GRAPHS_OFF, GRAPHS_AUTO, GRAPHS_ON = 0, 1, 2
MAT_FRICT, MAT_HERTZ = 0, 1
CP2_FRICT, CP2_HERTZ = 0, 1
ARITH_EXACT, ARITH_FMA, ARITH_DW = 0, 1, 2
LAW_IDEALELPL, LAW_HERTZ_DMT = 0, 1
UPDATE_PHYS_NEVER, UPDATE_PHYS_ALWAYS, UPDATE_PHYS_ONCE = 0, 1, 2

DOF_X, DOF_Y, DOF_Z, DOF_RX, DOF_RY, DOF_RZ = 1, 2, 4, 8, 16, 32
DOF_ALL = 63
CLUMP_CLUMPED, CLUMP_CLUMP = 64, 128
ENERGY_SKIP, GRAVITY_SKIP, TRACER_SKIP, DAMPING_SKIP = 256, 512, 1024, 2048

ENERGY_NAMES = ["kinetic", "grav", "nonviscDamp", "elast", "plast", "viscN", "viscT", "broken"]

D = C.POINTER(C.c_double)
I32 = C.POINTER(C.c_int32)
U32 = C.POINTER(C.c_uint32)
F32 = C.POINTER(C.c_float)


class Material(C.Structure):
    _fields_ = [("kind", C.c_int32), ("_pad", C.c_int32), ("density", C.c_double), ("young", C.c_double),
                ("ktDivKn", C.c_double), ("tanPhi", C.c_double), ("surfEnergy", C.c_double),
                ("alpha", C.c_double)]


class Params(C.Structure):
    _fields_ = [("dt", C.c_double), ("step", C.c_int64), ("gravity", C.c_double * 3), ("distFactor", C.c_double),
                ("loneMask", C.c_uint32), ("trackEnergy", C.c_int32),
                ("damping", C.c_double), ("reset", C.c_int32), ("kinSplit", C.c_int32),
                ("verletDist", C.c_double),
                ("noRatch", C.c_int32), ("iniLensTouch", C.c_int32), ("trsfRenorm", C.c_int32),
                ("approxMask", C.c_int32),
                ("updatePhys", C.c_int32), ("applyForces", C.c_int32), ("dist00", C.c_int32),
                ("cp2", C.c_int32), ("poisson", C.c_double), ("en", C.c_double),
                ("law", C.c_int32), ("noSlip", C.c_int32), ("noBreak", C.c_int32), ("noFrict", C.c_int32),
                ("iniEqlb", C.c_int32),
                ("relRollStiff", C.c_double), ("relTwistStiff", C.c_double), ("rollTanPhi", C.c_double),
                ("noAttraction", C.c_int32), ("_pad", C.c_int32),
                ("nMaterials", C.c_int32), ("_pad2", C.c_int32),
                ("materials", C.POINTER(Material)),
                ("ellSolver", C.c_int32), ("brentBits", C.c_int32), ("newtonTol", C.c_double),
                ("warmStart", C.c_int32), ("fallbackIters", C.c_int32), ("materialDt", C.POINTER(C.c_double)),
                ("dynDtPeriod", C.c_int32), ("_pad3", C.c_int32), ("dynDtMaxRelInc", C.c_double),
                ("dtSafety", C.c_double), ("arith", C.c_int32), ("_pad4", C.c_int32)]


class Particles(C.Structure):
    _fields_ = [("n", C.c_int32), ("_pad", C.c_int32), ("shape", I32), ("radius", D), ("wallAxis", I32),
                ("wallSense", I32), ("material", I32), ("mask", U32), ("flags", U32), ("mass", D),
                ("inertia", D), ("pos", D), ("ori", D), ("vel", D), ("angVel", D), ("force", D), ("torque", D),
                ("semiAxes", D), ("angMom", D), ("scene", I32), ("facetVerts", D), ("shaft", D)]


class Contacts(C.Structure):
    _fields_ = [("n", C.c_int64), ("idA", I32), ("idB", I32), ("real", I32), ("stepCreated", I32),
                ("minDist00Sq", D), ("trsf", D), ("contPt", D), ("geomOri", D), ("geomVel", D),
                ("geomAngVel", D), ("uN", D), ("force", D), ("torque", D), ("kn", D), ("kt", D), ("tanPhi", D),
                ("cellDist", I32)]


class LaunchShape(C.Structure):
    _fields_ = [("contactsBlock", C.c_int32), ("contactsPerSM", C.c_int32), ("cullBlock", C.c_int32),
                ("integratorBlock", C.c_int32), ("listsPerSM", C.c_int32), ("_pad", C.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if not k.startswith("_")}


class Cell(C.Structure):
    _fields_ = [("periodic", C.c_int32), ("homoDeform", C.c_int32), ("hSize", C.c_double * 9),
                ("trsf", C.c_double * 9), ("gradV", C.c_double * 9), ("nextGradV", C.c_double * 9),
                ("pprevHsize", C.c_double * 9)]


class Status(C.Structure):
    _fields_ = [("code", C.c_int32), ("detail", C.c_int32), ("step", C.c_int64), ("nContacts", C.c_int64),
                ("nReal", C.c_int64), ("nFullRuns", C.c_int64), ("capacity", C.c_int64),
                ("lastRunFull", C.c_int32), ("_pad", C.c_int32), ("ellSolves", C.c_int64), ("ellIters", C.c_int64),
                ("ellFallbacks", C.c_int64), ("dt", C.c_double), ("dynDtCrit", C.c_double), ("timeSum", C.c_double)]


EXPORTS = ["wdem_abi_version", "wdem_create", "wdem_destroy", "wdem_set_params", "wdem_upload_particles",
           "wdem_upload_contacts", "wdem_step", "wdem_download_particles", "wdem_contact_count",
           "wdem_download_contacts", "wdem_crit_dt", "wdem_get_energy", "wdem_reset_energy", "wdem_get_status",
           "wdem_last_error", "wdem_collide_boxes", "wdem_kernel_times", "wdem_set_timing", "wdem_set_queue_depth", "wdem_keep_geom",
           "wdem_make_cloud", "wdem_get_stream", "wdem_write_state", "wdem_read_state", "wdem_launch_count",
           "wdem_fp64_peak", "wdem_set_cell", "wdem_get_cell", "wdem_get_stress",
           "wdem_get_stress_noalloc", "wdem_warm_init", "wdem_warm_set_weights", "wdem_warm_get_weights",
           "wdem_warm_predict", "wdem_warm_grad", "wdem_warm_train", "wdem_ell_log", "wdem_ell_log_read", "wdem_make_cloud_radii", "wdem_set_contact_limit",
           "wdem_remove_particles", "wdem_add_particles", "wdem_set_launch_shape", "wdem_get_launch_shape",
           "wdem_autotune", "wdem_set_step_graphs", "wdem_graph_stats"]


def ptr(a, ctype):
    """ctypes pointer into a contiguous numpy array (or None)."""
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(ctype))


class ParticleArrays:
    """Host SoA buffers matching wdem_particles; keeps the numpy arrays alive."""

    def __init__(self, n):
        self.n = n
        self.shape = np.zeros(n, np.int32)
        self.radius = np.full(n, np.nan)
        self.wallAxis = np.zeros(n, np.int32)
        self.wallSense = np.zeros(n, np.int32)
        self.material = np.zeros(n, np.int32)
        self.mask = np.ones(n, np.uint32)
        self.flags = np.zeros(n, np.uint32)
        self.mass = np.zeros(n)
        self.inertia = np.zeros((n, 3))
        self.pos = np.zeros((n, 3))
        self.ori = np.zeros((n, 4)); self.ori[:, 0] = 1.0
        self.vel = np.zeros((n, 3))
        self.angVel = np.zeros((n, 3))
        self.force = np.zeros((n, 3))
        self.torque = np.zeros((n, 3))
        self.semiAxes = np.full((n, 3), np.nan)
        self.angMom = np.full((n, 3), np.nan)
        self.scene = np.zeros(n, np.int32)
        self.facetVerts = np.full((n, 9), np.nan)
        self.shaft = np.full(n, np.nan)

    def copy(self):
        o = ParticleArrays(self.n)
        for k, v in self.__dict__.items():
            if isinstance(v, np.ndarray):
                setattr(o, k, v.copy())
        return o

    def take(self, index):
        """The particles selected by `index` (integer indices), in that order."""
        idx = np.asarray(index, np.int64)
        o = ParticleArrays(len(idx))
        for k, v in self.__dict__.items():
            if isinstance(v, np.ndarray):
                setattr(o, k, np.ascontiguousarray(v[idx]))
        return o

    def struct(self):
        s = Particles()
        s.n = self.n
        s.shape = ptr(self.shape, C.c_int32); s.radius = ptr(self.radius, C.c_double)
        s.wallAxis = ptr(self.wallAxis, C.c_int32); s.wallSense = ptr(self.wallSense, C.c_int32)
        s.material = ptr(self.material, C.c_int32); s.mask = ptr(self.mask, C.c_uint32)
        s.flags = ptr(self.flags, C.c_uint32); s.mass = ptr(self.mass, C.c_double)
        s.inertia = ptr(self.inertia, C.c_double); s.pos = ptr(self.pos, C.c_double)
        s.ori = ptr(self.ori, C.c_double); s.vel = ptr(self.vel, C.c_double)
        s.angVel = ptr(self.angVel, C.c_double); s.force = ptr(self.force, C.c_double)
        s.torque = ptr(self.torque, C.c_double)
        s.semiAxes = ptr(self.semiAxes, C.c_double); s.angMom = ptr(self.angMom, C.c_double)
        s.scene = ptr(self.scene, C.c_int32)
        s.facetVerts = ptr(self.facetVerts, C.c_double)
        s.shaft = ptr(self.shaft, C.c_double)
        return s


class ContactArrays:
    """Host SoA buffers matching wdem_contacts."""

    def __init__(self, n):
        self.n = n
        self.idA = np.zeros(n, np.int32)
        self.idB = np.zeros(n, np.int32)
        self.real = np.zeros(n, np.int32)
        self.stepCreated = np.zeros(n, np.int32)
        self.minDist00Sq = np.zeros(n)
        self.trsf = np.zeros((n, 9))
        self.contPt = np.zeros((n, 3))
        self.geomOri = np.zeros((n, 4))
        self.geomVel = np.zeros((n, 3))
        self.geomAngVel = np.zeros((n, 3))
        self.uN = np.zeros(n)
        self.force = np.zeros((n, 3))
        self.torque = np.zeros((n, 3))
        self.kn = np.zeros(n)
        self.kt = np.zeros(n)
        self.tanPhi = np.zeros(n)
        self.cellDist = np.zeros((n, 3), np.int32)

    def struct(self):
        s = Contacts()
        s.n = self.n
        for name, ct in (("idA", C.c_int32), ("idB", C.c_int32), ("real", C.c_int32), ("stepCreated", C.c_int32),
                         ("cellDist", C.c_int32)):
            setattr(s, name, ptr(getattr(self, name), ct))
        for name in ("minDist00Sq", "trsf", "contPt", "geomOri", "geomVel", "geomAngVel", "uN", "force", "torque",
                     "kn", "kt", "tanPhi"):
            setattr(s, name, ptr(getattr(self, name), C.c_double))
        return s

    def keys(self):
        a = np.minimum(self.idA, self.idB).astype(np.int64)
        b = np.maximum(self.idA, self.idB).astype(np.int64)
        return (a << 32) | b

    def take(self, index):
        """The contacts selected by `index` (boolean mask or integer indices), in that order."""
        index = np.asarray(index)
        idx = np.nonzero(index)[0] if index.dtype == bool else index.astype(np.int64)
        o = ContactArrays(len(idx))
        for k, v in self.__dict__.items():
            if isinstance(v, np.ndarray):
                setattr(o, k, np.ascontiguousarray(v[idx]))
        return o

    def without_particles(self, ids):
        """The container after removing every contact of the given particles, as DemField::removeParticle
        does (src/dem/Particle.cpp:519-527); the other contacts keep their order and history."""
        ids = np.asarray(list(ids), np.int32)
        if len(ids) == 0 or self.n == 0:
            return self
        gone = np.isin(self.idA, ids) | np.isin(self.idB, ids)
        return self.take(~gone)


class WdemError(RuntimeError):
    """A wdem_* call failed; carries the negative WDEM_ERR_* code."""

    def __init__(self, code, msg):
        super().__init__(msg)
        self.code = code


_lib = None


def load(path=None):
    """Load libwdem.so (built in-tree by woo_gb300.build) and declare the ABI."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise RuntimeError(f"{p} is missing: the GB300 engine needs its CUDA library; run woo_gb300.build.build()")
    lib = C.CDLL(p)
    h = C.c_void_p
    sig = {
        "wdem_abi_version": ([], C.c_int),
        "wdem_create": ([C.c_int, C.c_int32, C.POINTER(h)], C.c_int),
        "wdem_destroy": ([h], C.c_int),
        "wdem_set_params": ([h, C.POINTER(Params)], C.c_int),
        "wdem_upload_particles": ([h, C.POINTER(Particles)], C.c_int),
        "wdem_upload_contacts": ([h, C.POINTER(Contacts)], C.c_int),
        "wdem_step": ([h, C.c_int32], C.c_int),
        "wdem_download_particles": ([h, C.POINTER(Particles)], C.c_int),
        "wdem_contact_count": ([h, C.POINTER(C.c_int64)], C.c_int),
        "wdem_download_contacts": ([h, C.POINTER(Contacts)], C.c_int),
        "wdem_crit_dt": ([h, C.POINTER(C.c_double)], C.c_int),
        "wdem_get_energy": ([h, C.POINTER(C.c_double), C.c_int32], C.c_int),
        "wdem_reset_energy": ([h], C.c_int),
        "wdem_get_status": ([h, C.POINTER(Status)], C.c_int),
        "wdem_last_error": ([h], C.c_char_p),
        "wdem_collide_boxes": ([h, C.c_int32, D, D, U32, C.c_uint32, I32, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
        "wdem_kernel_times": ([h, C.POINTER(C.c_char_p), D, I32, C.c_int32, I32], C.c_int),
        "wdem_set_timing": ([h, C.c_int32], C.c_int),
        "wdem_set_queue_depth": ([h, C.c_int32], C.c_int),
        "wdem_set_step_graphs": ([h, C.c_int32], C.c_int),
        "wdem_graph_stats": ([h, C.POINTER(C.c_int64), C.POINTER(C.c_int64)], C.c_int),
        "wdem_keep_geom": ([h, C.c_int32], C.c_int),
        "wdem_make_cloud": ([D, D, C.c_double, C.c_double, C.c_int64, C.c_uint64, C.c_int32, D, D], C.c_int64),
        "wdem_get_stream": ([h, C.POINTER(C.c_void_p)], C.c_int),
        "wdem_write_state": ([h, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "wdem_read_state": ([h, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p], C.c_int),
        "wdem_launch_count": ([h, C.POINTER(C.c_int64)], C.c_int),
        "wdem_fp64_peak": ([h, C.POINTER(C.c_double)], C.c_int),
        "wdem_set_cell": ([h, C.POINTER(Cell)], C.c_int),
        "wdem_get_cell": ([h, C.POINTER(Cell)], C.c_int),
        "wdem_get_stress": ([h, D], C.c_int),
        "wdem_get_stress_noalloc": ([h, D], C.c_int),
        "wdem_warm_init": ([h, C.c_uint64], C.c_int),
        "wdem_warm_set_weights": ([h, F32, C.c_int64], C.c_int),
        "wdem_warm_get_weights": ([h, F32, C.c_int64], C.c_int),
        "wdem_warm_predict": ([h, F32, C.c_int64, F32], C.c_int),
        "wdem_warm_grad": ([h, F32, C.c_int64, F32, F32], C.c_int),
        "wdem_warm_train": ([h, F32, C.c_int64, C.c_int32, C.c_int32, C.c_float, C.c_uint64, F32], C.c_int),
        "wdem_ell_log": ([h, C.c_int64], C.c_int),
        "wdem_make_cloud_radii": ([D, D, C.c_int32, C.c_int64, D, C.c_uint64, C.c_int32, D, D], C.c_int64),
        "wdem_set_contact_limit": ([h, C.c_int64], C.c_int),
        "wdem_remove_particles": ([h, C.c_int32, I32, D], C.c_int),
        "wdem_set_launch_shape": ([h, C.POINTER(LaunchShape)], C.c_int),
        "wdem_get_launch_shape": ([h, C.POINTER(LaunchShape)], C.c_int),
        "wdem_autotune": ([h, C.c_int32, C.POINTER(LaunchShape), C.POINTER(C.c_double), C.POINTER(C.c_double)], C.c_int),
        "wdem_add_particles": ([h, C.POINTER(Particles), I32], C.c_int),
        "wdem_ell_log_read": ([h, F32, C.c_int64, C.POINTER(C.c_int64)], C.c_int),
    }
    for name, (args, res) in sig.items():
        f = getattr(lib, name)
        f.argtypes = args
        f.restype = res
    if lib.wdem_abi_version() != ABI_VERSION:
        raise RuntimeError("libwdem.so ABI version mismatch; rebuild it")
    if path is None:
        _lib = lib
    return lib


class Handle:
    """One engine instance (one scene) on one CUDA device: a thin wrapper over the C ABI."""

    def __init__(self, max_particles, device=0):
        self.lib = load()
        self.h = C.c_void_p()
        rc = self.lib.wdem_create(device, int(max_particles), C.byref(self.h))
        if rc != 0:
            raise WdemError(rc, f"wdem_create failed ({rc}); is a CUDA device available?")

    def check(self, rc):
        if rc != 0:
            msg = self.lib.wdem_last_error(self.h)
            raise WdemError(rc, (msg.decode() if msg else "") or f"wdem error {rc}")
        return rc

    def close(self):
        if self.h:
            self.lib.wdem_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_params(self, params):
        self.check(self.lib.wdem_set_params(self.h, C.byref(params)))

    def upload_particles(self, pa):
        s = pa.struct()
        self.check(self.lib.wdem_upload_particles(self.h, C.byref(s)))

    def upload_contacts(self, ca):
        s = ca.struct()
        self.check(self.lib.wdem_upload_contacts(self.h, C.byref(s)))

    def step(self, n=1):
        self.check(self.lib.wdem_step(self.h, int(n)))

    def download_particles(self, pa):
        s = pa.struct()
        self.check(self.lib.wdem_download_particles(self.h, C.byref(s)))
        return pa

    def contact_count(self):
        n = C.c_int64()
        self.check(self.lib.wdem_contact_count(self.h, C.byref(n)))
        return n.value

    def download_contacts(self):
        ca = ContactArrays(self.contact_count())
        s = ca.struct()
        self.check(self.lib.wdem_download_contacts(self.h, C.byref(s)))
        return ca

    def crit_dt(self):
        v = C.c_double()
        self.check(self.lib.wdem_crit_dt(self.h, C.byref(v)))
        return v.value

    def status(self):
        st = Status()
        self.check(self.lib.wdem_get_status(self.h, C.byref(st)))
        return st

    def set_timing(self, on):
        self.check(self.lib.wdem_set_timing(self.h, 1 if on else 0))

    def remove_particles(self, ids, park=None):
        """Remove particles on the device (wdem_remove_particles): their slots become inert, their contacts
        die; `park` (k x 3) gives the positions the slots are parked at."""
        ids = np.ascontiguousarray(ids, np.int32)
        pk = None if park is None else np.ascontiguousarray(park, np.float64).reshape(len(ids), 3)
        self.check(self.lib.wdem_remove_particles(self.h, len(ids), ptr(ids, C.c_int32),
                                                  None if pk is None else ptr(pk, C.c_double)))

    def add_particles(self, particles, ids):
        """Insert particles on the device (wdem_add_particles) into the slots `ids`."""
        ids = np.ascontiguousarray(ids, np.int32)
        if len(ids) != particles.n:
            raise ValueError("one slot per added particle")
        s = particles.struct()
        self.check(self.lib.wdem_add_particles(self.h, C.byref(s), ptr(ids, C.c_int32)))

    def launch_shape(self):
        s = LaunchShape()
        self.check(self.lib.wdem_get_launch_shape(self.h, C.byref(s)))
        return s.as_dict()

    def set_launch_shape(self, **shape):
        s = LaunchShape()
        self.check(self.lib.wdem_get_launch_shape(self.h, C.byref(s)))
        for k, v in shape.items():
            setattr(s, k, int(v))
        self.check(self.lib.wdem_set_launch_shape(self.h, C.byref(s)))

    def autotune(self, steps_per_candidate=10):
        """Pick the fastest launch shape on the running simulation (wdem_autotune); returns
        dict(shape=..., ms=..., ms_start=...)."""
        s, a, b = LaunchShape(), C.c_double(), C.c_double()
        self.check(self.lib.wdem_autotune(self.h, int(steps_per_candidate), C.byref(s), C.byref(a), C.byref(b)))
        return {"shape": s.as_dict(), "ms": a.value, "ms_start": b.value}

    def set_contact_limit(self, max_contacts):
        """Upper bound on the contact container (0 = none): beyond it a step fails with WDEM_ERR_OVERFLOW."""
        self.check(self.lib.wdem_set_contact_limit(self.h, int(max_contacts)))

    def set_queue_depth(self, depth):
        """Steps queued before the host checks the collider trigger (1 = every step)."""
        self.check(self.lib.wdem_set_queue_depth(self.h, int(depth)))

    def set_step_graphs(self, mode):
        """How queued steps are launched: GRAPHS_OFF (kernel by kernel), GRAPHS_AUTO or GRAPHS_ON (one CUDA
        graph launch per queue, captured again when the launch arguments change)."""
        self.check(self.lib.wdem_set_step_graphs(self.h, int(mode)))

    def graph_stats(self):
        """(captures, replays) of queued-step graphs on this handle."""
        c, r = C.c_int64(), C.c_int64()
        self.check(self.lib.wdem_graph_stats(self.h, C.byref(c), C.byref(r)))
        return c.value, r.value

    def keep_geom(self, on):
        self.check(self.lib.wdem_keep_geom(self.h, 1 if on else 0))

    def kernel_times(self):
        names = (C.c_char_p * 8)()
        ms = (C.c_double * 8)()
        launches = (C.c_int32 * 8)()
        cnt = C.c_int32()
        self.check(self.lib.wdem_kernel_times(self.h, names, ms, launches, 8, C.byref(cnt)))
        return {names[i].decode(): (ms[i], launches[i]) for i in range(cnt.value)}

    def stream(self):
        v = C.c_void_p()
        self.check(self.lib.wdem_get_stream(self.h, C.byref(v)))
        return v.value

    def write_state(self, n, pos=None, vel=None, angVel=None, ori=None):
        """Addresses (ints) of host buffers, e.g. tensor.data_ptr() of pinned tensors, or None."""
        self.check(self.lib.wdem_write_state(self.h, int(n), pos, vel, angVel, ori))

    def read_state(self, n, pos=None, vel=None, angVel=None, ori=None):
        self.check(self.lib.wdem_read_state(self.h, int(n), pos, vel, angVel, ori))

    def energy(self):
        e = (C.c_double * 8)()
        self.check(self.lib.wdem_get_energy(self.h, e, 8))
        return dict(zip(ENERGY_NAMES, list(e)))

    def reset_energy(self):
        self.check(self.lib.wdem_reset_energy(self.h))

    def set_cell(self, hSize, trsf=None, gradV=None, nextGradV=None):
        c = Cell()
        c.periodic = 1
        c.homoDeform = 4
        for name, v in (("hSize", hSize), ("trsf", trsf if trsf is not None else np.eye(3)),
                        ("gradV", gradV if gradV is not None else np.zeros((3, 3))),
                        ("nextGradV", nextGradV if nextGradV is not None else np.zeros((3, 3)))):
            arr = getattr(c, name)
            for k, x in enumerate(np.asarray(v, float).reshape(9)):
                arr[k] = x
        self.check(self.lib.wdem_set_cell(self.h, C.byref(c)))

    def cell(self):
        c = Cell()
        self.check(self.lib.wdem_get_cell(self.h, C.byref(c)))
        return {k: np.array(list(getattr(c, k))).reshape(3, 3) for k in ("hSize", "trsf", "gradV", "nextGradV", "pprevHsize")}

    def stress(self):
        m = np.zeros(9)
        self.check(self.lib.wdem_get_stress(self.h, ptr(m, C.c_double)))
        return m.reshape(3, 3)

    def stress_noalloc(self):
        """wdem_get_stress through the allocation-free entry point (fixed device scratch)."""
        m = np.zeros(9)
        self.check(self.lib.wdem_get_stress_noalloc(self.h, ptr(m, C.c_double)))
        return m.reshape(3, 3)

    # ---- learned warm start of the ellipsoid solve
    def warm_init(self, seed=0):
        self.check(self.lib.wdem_warm_init(self.h, seed))

    def warm_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        self.check(self.lib.wdem_warm_set_weights(self.h, ptr(w, C.c_float), w.size))

    def warm_get_weights(self):
        w = np.zeros(WARM_NPARAM, np.float32)
        self.check(self.lib.wdem_warm_get_weights(self.h, ptr(w, C.c_float), w.size))
        return w

    def warm_predict(self, X):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.zeros((len(X), WARM_OUTPUTS), np.float32)
        self.check(self.lib.wdem_warm_predict(self.h, ptr(X, C.c_float), len(X), ptr(Y, C.c_float)))
        return Y

    def warm_grad(self, R):
        R = np.ascontiguousarray(R, np.float32)
        g = np.zeros(WARM_NPARAM, np.float32)
        loss = np.zeros(1, np.float32)
        self.check(self.lib.wdem_warm_grad(self.h, ptr(R, C.c_float), len(R), ptr(g, C.c_float), ptr(loss, C.c_float)))
        return g, float(loss[0])

    def warm_train(self, R, epochs=5, batch=512, lr=1e-3, seed=0):
        R = np.ascontiguousarray(R, np.float32)
        losses = np.zeros(max(epochs, 1), np.float32)
        self.check(self.lib.wdem_warm_train(self.h, ptr(R, C.c_float), len(R), epochs, batch, lr, seed,
                                            ptr(losses, C.c_float)))
        return losses[:epochs]

    def ell_log(self, cap):
        self.check(self.lib.wdem_ell_log(self.h, cap))

    def ell_log_read(self, cap):
        out = np.zeros((cap, WARM_RECORD), np.float32)
        n = C.c_int64()
        self.check(self.lib.wdem_ell_log_read(self.h, ptr(out, C.c_float), cap, C.byref(n)))
        return out[:n.value]

    def fp64_peak(self):
        v = C.c_double()
        self.check(self.lib.wdem_fp64_peak(self.h, C.byref(v)))
        return v.value

    def launch_count(self):
        v = C.c_int64()
        self.check(self.lib.wdem_launch_count(self.h, C.byref(v)))
        return v.value

    def collide_boxes(self, mins, maxs, mask, lone_mask):
        mins = np.ascontiguousarray(mins, np.float64)
        maxs = np.ascontiguousarray(maxs, np.float64)
        mask = np.ascontiguousarray(mask, np.uint32)
        n = len(mins)
        npairs = C.c_int64()
        self.check(self.lib.wdem_collide_boxes(self.h, n, ptr(mins, C.c_double), ptr(maxs, C.c_double),
                                               ptr(mask, C.c_uint32), int(lone_mask), None, 0, C.byref(npairs)))
        pairs = np.zeros((max(npairs.value, 1), 2), np.int32)
        self.check(self.lib.wdem_collide_boxes(self.h, n, ptr(mins, C.c_double), ptr(maxs, C.c_double),
                                               ptr(mask, C.c_uint32), int(lone_mask), ptr(pairs, C.c_int32),
                                               npairs.value, C.byref(npairs)))
        return pairs[:npairs.value]


def make_cloud(lo, hi, rmin, rmax, n, seed, max_attempts=200):
    """Seeded non-overlapping sphere cloud (see wdem_make_cloud); returns (centers (k,3), radii (k,))."""
    lib = load()
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    centers = np.zeros((n, 3))
    radii = np.zeros(n)
    k = lib.wdem_make_cloud(ptr(lo, C.c_double), ptr(hi, C.c_double), float(rmin), float(rmax), int(n), int(seed),
                            int(max_attempts), ptr(centers, C.c_double), ptr(radii, C.c_double))
    if k < 0:
        raise WdemError(int(k), "wdem_make_cloud: bad arguments")
    return centers[:k].copy(), radii[:k].copy()


def make_cloud_radii(lo, hi, radii_in, seed, periodic=False, max_attempts=200):
    """Seeded non-overlapping cloud for given radii (see wdem_make_cloud_radii); returns (centers, radii)."""
    lib = load()
    lo = np.ascontiguousarray(lo, np.float64)
    hi = np.ascontiguousarray(hi, np.float64)
    rin = np.ascontiguousarray(radii_in, np.float64)
    n = len(rin)
    centers = np.zeros((n, 3))
    radii = np.zeros(n)
    k = lib.wdem_make_cloud_radii(ptr(lo, C.c_double), ptr(hi, C.c_double), 1 if periodic else 0, n, ptr(rin, C.c_double),
                                  int(seed), int(max_attempts), ptr(centers, C.c_double), ptr(radii, C.c_double))
    if k < 0:
        raise WdemError(int(k), "wdem_make_cloud_radii: bad arguments")
    return centers[:k].copy(), radii[:k].copy()
