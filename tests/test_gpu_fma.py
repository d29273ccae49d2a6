"""The contracted arithmetic variants (wdem_params.arith = WDEM_ARITH_FMA, and WDEM_ARITH_DW with the contact
law of real sphere and wall contacts in double-word FP32) against the exact one.

Tolerances (the ones the engine promises for this variant):
- after one step from an identical state (particles and contacts with history uploaded to both), every
  real contact's force (FrictPhys / HertzPhys force in the contact frame) within 1e-12 relative of the
  exact variant's, |dF| <= 1e-12 |F| (contacts whose force is below 1e-9 of the largest are compared at
  1e-12 of the largest force instead: they are breaking or just forming), the same real contacts, and
  particle forces and torques within 1e-12 relative of the largest;
- over long runs, the kinetic-energy trace and the energy balance agree statistically: the variants'
  trajectories part by rounding (granular flow amplifies differences), so the traces are compared as
  time series of a bulk quantity, within 1 % of the trace's scale at every sample and 0.2 % on average,
  and the energy-balance error of the contracted run is no larger than twice the exact run's plus 1e-3
  of the energy scale.
"""
import numpy as np
import pytest

from woo_gb300 import abi, scenes

from helpers import gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def _state(law, seed):
    spec = scenes.random_cloud(4000, seed, box=(0.2, 0.2, 0.2), rmin=0.003, rmax=0.005, dense=0.7, law=law,
                               vel_scale=0.05, angvel_scale=1.0)
    h = gpu_handle(spec, keep_geom=False)
    h.step(120)
    pa = h.download_particles(spec.particles.copy())
    ca = h.download_contacts()
    step = h.status().step
    h.close()
    return spec, pa, ca, step


def _handle(spec, pa, ca, step, arith):
    p = scenes.copy_params(spec.params)
    p.step = step
    p.arith = arith
    h = abi.Handle(pa.n)
    h.keep_geom(False)
    h.set_params(p)
    h.upload_particles(pa)
    h.set_params(p)
    h.upload_contacts(ca)
    return h


def _compare_one_step(he, hf, pa):
    ce, cf = he.download_contacts(), hf.download_contacts()
    re, rf = ce.real == 1, cf.real == 1
    assert np.array_equal(ce.keys()[re], cf.keys()[rf]), "real contact sets differ"
    Fe, Ff = ce.force[re], cf.force[rf]
    ne = np.linalg.norm(Fe, axis=1)
    d = np.linalg.norm(Ff - Fe, axis=1)
    big = ne >= 1e-9 * ne.max()
    assert big.sum() > 500
    rel = d[big] / ne[big]
    assert rel.max() <= 1e-12, f"max relative force difference {rel.max():.3g}"
    assert (d[~big] <= 1e-12 * ne.max()).all()
    pe, pf = gpu_particles(he, pa.n), gpu_particles(hf, pa.n)
    for name in ("force", "torque"):
        a, b = getattr(pe, name), getattr(pf, name)
        assert np.allclose(a, b, rtol=0, atol=1e-12 * np.abs(a).max()), name
    # positions after the step: the update is never contracted, the velocities differ by rounding only
    assert np.allclose(pe.pos, pf.pos, rtol=0, atol=1e-15)
    he.close()
    hf.close()


@pytest.mark.parametrize("arith", ["fma", "dw"])
@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_one_step_contact_forces(wdem_lib, law, arith):
    spec, pa, ca, step = _state(law, 21)
    assert int(ca.real.sum()) > 500
    he = _handle(spec, pa, ca, step, abi.ARITH_EXACT)
    hf = _handle(spec, pa, ca, step, abi.ARITH_FMA if arith == "fma" else abi.ARITH_DW)
    he.step(1)
    hf.step(1)
    _compare_one_step(he, hf, pa)


@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_one_step_contact_forces_periodic_dw(wdem_lib, law):
    """The double-word law on a sheared periodic packing (image shifts and shift velocities of pB)."""
    spec = scenes.periodic_cloud(3000, 4, law=law, shear=0.5)
    h = gpu_handle(spec, keep_geom=False)
    h.step(150)
    pa = h.download_particles(spec.particles.copy())
    ca = h.download_contacts()
    cl = h.cell()
    cell = {k: cl[k] for k in ("hSize", "trsf", "gradV", "nextGradV")}
    step = h.status().step
    h.close()
    assert int(ca.real.sum()) > 500
    hs = []
    for arith in (abi.ARITH_EXACT, abi.ARITH_DW):
        p = scenes.copy_params(spec.params)
        p.step = step
        p.arith = arith
        hh = abi.Handle(pa.n)
        hh.keep_geom(False)
        hh.set_params(p)
        hh.upload_particles(pa)
        hh.set_params(p)
        hh.set_cell(**cell)
        hh.upload_contacts(ca)
        hh.step(1)
        hs.append(hh)
    _compare_one_step(hs[0], hs[1], pa)


def test_dw_long_run_kinetic(wdem_lib):
    """Without energy tracking (which keeps the FP64 law): the kinetic energy of the particles, sampled every
    100 steps over 3000 steps of a dense Hertz-DMT packing settling under gravity, agrees between the exact
    and the double-word runs within 1 % of the trace's scale at every sample and 0.2 % on average."""
    traces = {}
    for arith in (abi.ARITH_EXACT, abi.ARITH_DW):
        spec = scenes.random_cloud(4000, 5, box=(0.25, 0.25, 0.25), rmin=0.003, rmax=0.005, dense=0.9, law="hertz",
                                   arith=arith)
        h = gpu_handle(spec, keep_geom=False)
        m = spec.particles.mass
        ek = []
        for _ in range(30):
            h.step(100)
            v = gpu_particles(h, spec.particles.n).vel
            ek.append(0.5 * float(np.sum(m * np.sum(v * v, axis=1))))
        traces[arith] = np.array(ek)
        h.close()
    a, b = traces[abi.ARITH_EXACT], traces[abi.ARITH_DW]
    scale = a.max()
    assert scale > 0
    assert np.abs(a - b).max() <= 0.01 * scale
    assert np.abs(a - b).mean() <= 0.002 * scale


@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_long_run_energy_statistics(wdem_lib, law):
    traces, balance = {}, {}
    for arith in (abi.ARITH_EXACT, abi.ARITH_FMA):
        spec = scenes.random_cloud(4000, 5, box=(0.25, 0.25, 0.25), rmin=0.003, rmax=0.005, dense=0.9, law=law,
                                   trackEnergy=1, arith=arith)
        h = gpu_handle(spec, keep_geom=False)
        ek, tot = [], []
        for _ in range(30):
            h.step(100)
            e = h.energy()
            ek.append(e["kinetic"])
            tot.append(sum(e[k] for k in abi.ENERGY_NAMES if k != "kinetic") + e["kinetic"])
        traces[arith] = np.array(ek)
        balance[arith] = np.array(tot)
        h.close()
    a, b = traces[abi.ARITH_EXACT], traces[abi.ARITH_FMA]
    scale = a.max()
    assert scale > 0
    assert np.abs(a - b).max() <= 0.01 * scale
    assert np.abs(a - b).mean() <= 0.002 * scale
    escale = np.abs(balance[abi.ARITH_EXACT]).max() + scale
    err_e = np.ptp(balance[abi.ARITH_EXACT])
    err_f = np.ptp(balance[abi.ARITH_FMA])
    assert err_f <= 2 * err_e + 1e-3 * escale, (err_e, err_f)
