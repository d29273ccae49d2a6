"""Capsules on the GPU (Cg2_Sphere_Capsule_L6Geom, Cg2_Wall_Capsule_L6Geom, Cg2_Capsule_Capsule_L6Geom,
Bo1_Capsule_Aabb) against the oracle:

- the known-answer placements of the oracle's capsule test after one step: contacts bit-exact;
- 300 capsules and 300 spheres, overlapping at the start, in a walled box under gravity for 1500 steps:
  positions, velocities, forces and torques bit-exact, contacts and their history bit-exact;
  orientations and angular velocities of the aspherical Leapfrog within 1e-12 (sin/cos of CUDA and
  of the C library may differ in the last bit), as for ellipsoids;
- a capsule scene through the Python surface (Capsule.make, minimalEngines);
- the refusals: a capsule in a periodic cell, a facet whose mask meets capsules."""
import math

import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, dem, scenes

from helpers import assert_same_contacts, gpu_handle, gpu_particles
from test_oracle_capsule import R, capsule_scene, quat_z

pytestmark = pytest.mark.gpu


def assert_capsule_state(pg, po, tol=1e-12):
    for name in ("pos", "vel", "force"):
        a, b = getattr(pg, name), getattr(po, name)
        assert np.array_equal(a, b), f"{name} differs at {np.argwhere(a != b)[:5].tolist()}"
    for name in ("angVel", "torque", "ori"):
        a, b = getattr(pg, name), getattr(po, name)
        scale = max(1.0, float(np.max(np.abs(b))))
        assert np.allclose(a, b, rtol=0, atol=tol * scale), f"{name} differs beyond {tol}"


PLACEMENTS = [
    ([((0, 0, 0), (1, 0, 0, 0))], [((.03, .029, 0), 0.01)], []),
    ([((0, 0, 0), (1, 0, 0, 0))], [((.07, .0205, 0), 0.01)], []),
    ([((.1, .2, .019), (1, 0, 0, 0))], [], [(2, 1, 0.0)]),
    ([((.1, .2, .032), scenes.quat_from_axis_angle((0, 1, 0), 0.3))], [], [(2, 1, 0.0)]),
    ([((0, 0, 0), (1, 0, 0, 0)), ((0, 0, .039), quat_z(math.pi / 2))], [], []),
    ([((0, 0, 0), (1, 0, 0, 0)), ((0, .039, 0), (1, 0, 0, 0))], [], []),
    ([((0, 0, 0), (1, 0, 0, 0)), ((.06, .039, 0), (1, 0, 0, 0))], [], []),
]


@pytest.mark.parametrize("k", range(len(PLACEMENTS)))
def test_known_placements(wdem_lib, k):
    caps, spheres, walls = PLACEMENTS[k]
    spec = capsule_scene(caps, spheres=spheres, walls=walls)
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    h.step(1)
    o.step(1)
    cg, co = h.download_contacts(), o.contacts()
    assert cg.n >= 1 and cg.real.sum() == 1
    assert_same_contacts(cg, co)
    assert np.array_equal(cg.uN, co.uN)
    assert_capsule_state(gpu_particles(h, spec.particles.n), o.particles())
    h.close()


def test_capsule_cloud(wdem_lib):
    spec = scenes.capsule_cloud(300, 300, 3)
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    n = spec.particles.n
    shape = spec.particles.shape
    kinds = set()
    for block in (1, 49, 250, 400, 800):
        h.step(block)
        o.step(block)
        cg, co = h.download_contacts(), o.contacts()
        assert_capsule_state(gpu_particles(h, n), o.particles())
        assert_same_contacts(cg, co)
        r = cg.real == 1
        kinds |= {(int(a), int(b)) for a, b in zip(shape[cg.idA[r]], shape[cg.idB[r]])}
    # sphere-capsule, capsule-capsule and wall-capsule contacts were all compared
    assert {(abi.SHAPE_SPHERE, abi.SHAPE_CAPSULE), (abi.SHAPE_CAPSULE, abi.SHAPE_CAPSULE),
            (abi.SHAPE_WALL, abi.SHAPE_CAPSULE)} <= kinds
    h.close()


def test_scene_api(wdem_lib):
    """Capsules dropped on a wall through the Python surface: the trajectories equal the oracle's."""
    from woo_gb300 import utils
    from woo_gb300.core import Scene
    m = dem.FrictMat(density=2000, young=1e7, ktDivKn=0.2, tanPhi=0.5)
    par = [utils.wall(0, axis=2, sense=1, mat=m)]
    par += [utils.capsule((0.05 * k, 0.01 * k, 0.03 + 0.01 * k), 0.01, 0.02 + 0.005 * k,
                          ori=scenes.quat_from_axis_angle((1, 1, 0), 0.4 * k), mat=m) for k in range(6)]
    S = Scene(fields=[dem.DemField(gravity=(0, 0, -9.81), par=par)],
              engines=dem.DemField.minimalEngines(damping=0.3, dynDtPeriod=0), dtSafety=0.5)
    S._prepare_dt()
    g = S._engine()
    params = g._build_params(S, S.dem)
    pa = g._pack(S.dem)
    o = bridge.Oracle(params, pa)
    S.run(4000)
    o.step(4000)
    po = o.particles()
    for p in S.dem.par:
        if isinstance(p.shape, dem.Capsule):
            assert np.array_equal(p.pos, po.pos[p.id])
            assert np.allclose(p.ori, po.ori[p.id], rtol=0, atol=1e-12)
    assert len(S.dem.con) == o.contacts().n


def test_refusals(wdem_lib):
    spec = capsule_scene([((0, 0, 0), (1, 0, 0, 0))])
    h = abi.Handle(spec.particles.n)
    h.set_params(spec.params)
    h.set_cell(np.eye(3))
    with pytest.raises(abi.WdemError, match="periodic") as ei:
        h.upload_particles(spec.particles)
    assert ei.value.code == abi.WDEM_ERR_UNSUPPORTED
    h.close()
    spec = capsule_scene([((0, 0, .5), (1, 0, 0, 0))])
    pa = scenes.add_facets(spec.particles, [((0, 0, 0), (1, 0, 0), (0, 1, 0))])
    pa.mask[-1] = dem.DEFAULT_MOVABLE_MASK  # shares the capsule's bits outside loneMask
    h = abi.Handle(pa.n)
    h.set_params(spec.params)
    h.upload_particles(pa)
    with pytest.raises(abi.WdemError, match="facet-capsule") as ei:
        h.step(1)
    assert ei.value.code == abi.WDEM_ERR_UNSUPPORTED
    h.close()
