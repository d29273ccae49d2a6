"""Shared helpers for the parity tests: run the same scene through the GPU engine and the oracle."""
import numpy as np

from woo_gb300 import abi


def gpu_handle(spec, keep_geom=True, contacts=None):
    h = abi.Handle(max(spec.particles.n, 1))
    h.keep_geom(keep_geom)
    h.set_params(spec.params)
    h.upload_particles(spec.particles)
    h.set_params(spec.params)
    if getattr(spec, "cell", None) is not None:
        h.set_cell(**spec.cell)
    if contacts is not None:
        h.upload_contacts(contacts)
    return h


def gpu_particles(h, n):
    return h.download_particles(abi.ParticleArrays(n))


def assert_same_contacts(cg, co, exact=True, rtol=1e-12):
    """Contact containers equal: same pairs (sorted by key), same orientation and state; history equal
    bitwise (exact) or within rtol relative to each quantity's scale."""
    assert cg.n == co.n, f"contact count {cg.n} != {co.n}"
    kg, ko = cg.keys(), co.keys()
    assert np.array_equal(kg, ko), "pair sets differ"
    assert np.array_equal(cg.idA, co.idA) and np.array_equal(cg.idB, co.idB), "orientation differs"
    assert np.array_equal(cg.real, co.real), "real flags differ"
    assert np.array_equal(cg.stepCreated, co.stepCreated), "stepCreated differs"
    r = cg.real.astype(bool)
    for name in ("trsf", "contPt", "force", "kn", "kt", "tanPhi", "geomOri"):
        a, b = getattr(cg, name)[r], getattr(co, name)[r]
        if exact:
            bad = ~((a == b) | (np.isnan(a) & np.isnan(b)))
            assert not bad.any(), f"{name} differs bitwise at {np.argwhere(bad)[:5].tolist()}: {a[bad][:5]} vs {b[bad][:5]}"
        else:
            scale = np.max(np.abs(b)) if b.size else 1.0
            assert np.allclose(a, b, rtol=rtol, atol=rtol * scale), f"{name} differs beyond {rtol}"


def assert_same_particles(pg, po, exact=True, rtol=1e-12, ori_tol=1e-12):
    for name in ("pos", "vel", "angVel", "force", "torque"):
        a, b = getattr(pg, name), getattr(po, name)
        if exact:
            bad = a != b
            assert not bad.any(), f"{name} differs bitwise at {np.argwhere(bad)[:5].tolist()}: {a[bad][:5]} vs {b[bad][:5]}"
        else:
            scale = np.max(np.abs(b)) if b.size else 1.0
            assert np.allclose(a, b, rtol=rtol, atol=rtol * scale), f"{name} differs beyond {rtol}"
    # sin/cos of CUDA and of the C library may differ in the last bit: orientation compared with a tolerance
    assert np.allclose(pg.ori, po.ori, rtol=0, atol=ori_tol), "ori differs"


def assert_same_real_contacts(cg, co):
    """Real contacts equal bitwise (pairs, orientation, history).  Potential pairs may differ after a contact
    container was uploaded: the reference's initial sort keeps uploaded potential pairs whose boxes do not
    meet along the sort axis, the engine's rebuild drops every pair whose boxes do not overlap; neither
    carries physics."""
    rg, ro = cg.real == 1, co.real == 1
    assert_same_contacts(cg.take(rg), co.take(ro))
