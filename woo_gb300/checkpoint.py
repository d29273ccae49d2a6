"""Engine state checkpoints: particles, the contact container with its history, the periodic cell and
the step/dt, in a versioned numpy archive.

The reference saves whole scenes through its object serialization (Scene.save, ObjectIO.hpp:12-75)
and rebuilds the collider's arrays after loading (a full collider run: contacts->dirty,
InsertionSortCollider.hpp:225).  This format holds what the GPU engine needs to continue a run: the
wdem_particles and wdem_contacts arrays of woo_gb300.abi, the cell matrices, Scene.step and Scene.dt.
After `resume` the first step runs the collider in full, as the reference does after a load, so real
contacts, their history and the particle trajectories continue exactly; potential (not touching)
pairs are found anew.  The ellipsoid solver's last maximiser (a warm start only) is not saved, nor is
Cell.pprevHsize: every step starts with Cell::integrateAndUpdate (src/core/Scene.cpp:411), which sets it
from the previous and new hSize before the contact loop reads it, so a sheared periodic run resumes bit
for bit without it.
"""
import numpy as np

from . import abi

FORMAT = "wdem-state"
VERSION = 1


def save_state(path, particles, contacts, step, dt, cell=None):
    """Write one state to `path` (a .npz archive)."""
    data = {"format": np.array(FORMAT), "version": np.array(VERSION), "step": np.array(int(step)),
            "dt": np.array(float(dt)), "n": np.array(particles.n), "nc": np.array(contacts.n)}
    for k, v in particles.__dict__.items():
        if isinstance(v, np.ndarray):
            data["p_" + k] = v
    for k, v in contacts.__dict__.items():
        if isinstance(v, np.ndarray):
            data["c_" + k] = v
    if cell is not None:
        for k in ("hSize", "trsf", "gradV", "nextGradV"):
            data["cell_" + k] = np.asarray(cell[k], np.float64).reshape(3, 3)
    np.savez_compressed(path, **data)


def load_state(path):
    """Read a state written by save_state: dict(particles=ParticleArrays, contacts=ContactArrays, step,
    dt, cell=dict or None)."""
    with np.load(path, allow_pickle=False) as z:
        if str(z["format"]) != FORMAT:
            raise ValueError(f"{path}: not a {FORMAT} archive")
        if int(z["version"]) != VERSION:
            raise ValueError(f"{path}: {FORMAT} version {int(z['version'])}, this reader knows {VERSION}")
        pa = abi.ParticleArrays(int(z["n"]))
        for k in pa.__dict__:
            if "p_" + k in z:
                setattr(pa, k, z["p_" + k].copy())
        ca = abi.ContactArrays(int(z["nc"]))
        for k in ca.__dict__:
            if "c_" + k in z:
                setattr(ca, k, z["c_" + k].copy())
        cell = None
        if "cell_hSize" in z:
            cell = {k: z["cell_" + k].copy() for k in ("hSize", "trsf", "gradV", "nextGradV")}
        return dict(particles=pa, contacts=ca, step=int(z["step"]), dt=float(z["dt"]), cell=cell)


def checkpoint(handle, path, static):
    """Save a running GPU handle: its dynamic state merged into `static` (the ParticleArrays it was
    created from: shapes, radii, materials, masses), its contacts, cell, step and dt."""
    pa = static.copy()
    handle.download_particles(pa)
    st = handle.status()
    cell = handle.cell() if _periodic(handle) else None
    save_state(path, pa, handle.download_contacts(), st.step, st.dt, cell)


def resume(path, params, device=0):
    """A new GPU handle continuing the saved state with engine parameters `params` (wdem_params; their
    step and dt are taken from the archive)."""
    s = load_state(path)
    params.step = s["step"]
    params.dt = s["dt"]
    h = abi.Handle(max(s["particles"].n, 1), device=device)
    h.set_params(params)
    h.upload_particles(s["particles"])
    h.set_params(params)
    if s["cell"] is not None:
        h.set_cell(**s["cell"])
    h.upload_contacts(s["contacts"])
    return h


def _periodic(handle):
    c = abi.Cell()
    handle.check(handle.lib.wdem_get_cell(handle.h, abi.C.byref(c)))
    return bool(c.periodic)
