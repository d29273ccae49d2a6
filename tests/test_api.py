"""The Woo-compatible Python surface (no GPU needed): scene construction, engine lists, labels,
attribute mapping into the engine parameters, critical dt, and loud failure without a CUDA device."""
import math

import numpy as np
import pytest

import woo_gb300 as woo
from woo_gb300 import abi, dem, utils
from woo_gb300.core import Scene


def small_scene(**kw):
    m = dem.FrictMat(density=2500, young=1e7, ktDivKn=0.2, tanPhi=0.5)
    par = [dem.Wall.make(0, axis=2, sense=1, mat=m)] + [dem.Sphere.make((0, 0, 0.011 + 0.021 * k), 0.01, mat=m) for k in range(5)]
    return Scene(fields=[dem.DemField(gravity=(0, 0, -9.81), par=par)],
                 engines=dem.DemField.minimalEngines(damping=0.2, dynDtPeriod=0), **kw)


def test_minimal_engines_structure():
    ee = utils.defaultEngines(dynDtPeriod=0)
    assert [type(e).__name__ for e in ee] == ["Leapfrog", "InsertionSortCollider", "ContactLoop"]
    assert ee[0].reset is True and ee[1].verletDist == -0.05
    assert isinstance(ee[2].phyFunctors[0], dem.Cp2_FrictMat_FrictPhys)
    assert isinstance(ee[2].lawFunctors[0], dem.Law2_L6Geom_FrictPhys_IdealElPl)
    assert type(utils.defaultEngines()[-1]).__name__ == "DynDt"


def test_labels_and_attributes():
    S = small_scene()
    assert isinstance(S.lab.contactLoop, dem.ContactLoop)
    assert isinstance(S.lab.contactLaw, dem.Law2_L6Geom_FrictPhys_IdealElPl)
    S.lab.contactLoop.updatePhys = "always"
    g = dem.GpuDemEngine.fromEngines(S.engines)
    assert g.updatePhys == "always" and g.damping == 0.2 and g.verletDist == -0.05
    with pytest.raises(AttributeError):
        dem.FrictMat(yuong=1)


def test_particle_construction_matches_woo_formulas():
    m = dem.FrictMat(density=3000)
    p = dem.Sphere.make((1, 2, 3), 0.005, mat=m)
    mass = ((4 / 3.0) * math.pi) * (0.005 ** 3) * 3000
    assert p.mass == pytest.approx(mass, rel=1e-15)
    assert np.allclose(p.inertia, 0.4 * mass * 0.005 ** 2)
    w = dem.Wall.make(0.5, axis=1, sense=-1)
    assert w.blocked == "xyzXYZ" and w.mask == dem.DemField.defaultBoundaryMask
    assert np.array_equal(w.pos, [0, 0.5, 0])


def test_crit_dt_and_auto_dt():
    S = small_scene(dtSafety=0.4)
    pw = 0.01 / math.sqrt(1e7 / 2500)
    assert S.dem.critDt() == pytest.approx(pw)
    S._prepare_dt()
    assert S.dt == pytest.approx(0.4 * pw)


def test_params_packing():
    S = small_scene()
    S._prepare_dt()
    g = S._engine()
    p = g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    assert p.law == abi.LAW_IDEALELPL and p.cp2 == abi.CP2_FRICT and p.reset == 1
    assert p.loneMask == 2 and list(p.gravity) == [0, 0, -9.81]
    assert pa.n == 6 and pa.shape[0] == abi.SHAPE_WALL and pa.flags[0] == 63
    assert pa.mask[1] == 5 and pa.wallAxis[0] == 2 and pa.wallSense[0] == 1


def test_unsupported_engine_rejected():
    class PyRunner(dem.Engine):
        pass
    S = small_scene()
    S.engines = utils.defaultEngines(dynDtPeriod=0) + [PyRunner()]
    with pytest.raises(RuntimeError, match="PyRunner"):
        S.run(1)


def test_dyndt_engine_is_taken_over():
    S = small_scene()
    S.engines = utils.defaultEngines(dynDtPeriod=100)
    g = S._engine()
    assert isinstance(g._dynDt, dem.DynDt) and g._dynDt.stepPeriod == 100 and g._dynDt.maxRelInc == 1e-4


def test_fails_loudly_without_gpu():
    from conftest import HAS_GPU
    if HAS_GPU:
        pytest.skip("a GPU is present")
    S = small_scene()
    with pytest.raises(RuntimeError):
        S.run(1)


def test_guess_moving():
    """py/tests/test_demfield.py:11-22 (testGuessMoving)."""
    def dd(blocked="", mass=0.0, vel=(0, 0, 0)):
        n = dem.Node()
        n.dem.blocked = blocked
        n.dem.mass = mass
        n.dem.vel = vel
        return n.dem
    assert not dd(mass=0).guessMoving()
    assert not dd("xyz", mass=0).guessMoving()
    assert dd("xyzXY", mass=1).guessMoving()
    assert not dd("xyzXYZ", mass=1).guessMoving()
    assert dd("xyzXYZ", mass=1, vel=(1, 1, 1)).guessMoving()


def test_nodes_left_out_are_held_fixed():
    """A particle whose node is not collected into DemField.nodes (nodes=False, or nodes=-1 and
    guessMoving() false) is not integrated: the engine uploads it fully blocked and at rest, while the
    Python side keeps its own attributes."""
    m = dem.FrictMat()
    S = small_scene()
    ghost = dem.Sphere.make((0, 0, 0.5), 0.01, mat=m)
    ghost.shape.nodes[0].dem.mass = 0.0
    S.dem.par.add(ghost)
    held = dem.Sphere.make((0, 0, 0.8), 0.01, mat=m)
    S.dem.par.add(held, nodes=False)
    held.vel = (1, 2, 3)
    S._prepare_dt()
    g = S._engine()
    g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    dv = g._device_view(S.dem, pa)
    for p in (ghost, held):
        assert dv.flags[p.id] & 63 == 63 and not dv.vel[p.id].any()
    assert pa.flags[held.id] & 63 == 0 and tuple(pa.vel[held.id]) == (1, 2, 3)
    others = [p.id for p in S.dem.par if p.id not in (ghost.id, held.id)]
    assert np.array_equal(dv.flags[others], pa.flags[others])


def test_impose_is_rejected_not_ignored():
    """DemData.impose (prescribed motion inside Leapfrog) is not provided: setting one raises."""
    p = dem.Sphere.make((0, 0, 0), 0.01)
    assert p.impose is None
    p.impose = None
    with pytest.raises(RuntimeError, match="impose"):
        p.impose = object()


def test_exec_time_with_timing_enabled(monkeypatch):
    """Master.timingEnabled: execTime/execCount on the engine and on Woo's trio it stands for."""
    from oracle_handle import run_on_oracle
    S = small_scene()
    run_on_oracle(monkeypatch, S, 5)
    assert S.lab.contactLoop.execCount == 0
    woo.master.timingEnabled = True
    try:
        run_on_oracle(monkeypatch, S, 7)
    finally:
        woo.master.timingEnabled = False
    run_on_oracle(monkeypatch, S, 3)
    for e in (S.lab.leapfrog, S.lab.collider, S.lab.contactLoop):
        assert e.execCount == 7
    assert S.lab.contactLoop.execTime > 0 and S._gpu.execCount == 7
    assert S._gpu.execTime >= S.lab.contactLoop.execTime


def test_unbalanced_force_and_energy(monkeypatch):
    """DemFuncs::unbalancedForce and utils.unbalancedEnergy on a settling column (on the oracle): the
    ratio falls as the column comes to rest, and matches the definition recomputed here."""
    from oracle_handle import run_on_oracle
    S = small_scene(trackEnergy=True)
    run_on_oracle(monkeypatch, S, 50)
    assert math.isnan(S.dem.unbalancedForce())            # no contact yet: 0/0, as in the reference
    run_on_oracle(monkeypatch, S, 500)
    u0 = S.dem.unbalancedForce()
    assert math.isfinite(u0)
    run_on_oracle(monkeypatch, S, 4000)
    u1 = S.dem.unbalancedForce()
    assert u1 < u0
    F = [np.linalg.norm(p.f) for p in S.dem.par if p.blocked == ""]
    C = [np.linalg.norm(c.phys.force) for c in S.dem.con]
    assert u1 == pytest.approx(np.mean(F) / np.mean(C), rel=1e-12)
    assert S.dem.unbalancedForce(useMaxForce=True) == pytest.approx(max(F) / np.mean(C), rel=1e-12)
    assert utils.unbalancedForce(S) == u1
    ue = utils.unbalancedEnergy(S)
    e = S.energy
    assert ue == e["kinetic"] / e["elast"]


def test_demfield_nodes_are_the_integrated_ones():
    S = small_scene()
    ids = [n._local["pos"][2] for n in S.dem.nodes]
    assert len(S.dem.nodes) == 5 and min(ids) > 0         # the wall (fixed, massless) is not collected


def test_particle_kinetic_energies():
    p = dem.Sphere.make((0, 0, 0), 0.01, vel=(1, 2, 2))
    p.angVel = (0, 0, 3)
    assert p.Ekt == pytest.approx(0.5 * p.mass * 9)
    assert p.Ekr == pytest.approx(0.5 * p.inertia[2] * 9)
    assert p.Ek == pytest.approx(p.Ekt + p.Ekr)
