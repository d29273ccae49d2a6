"""Launch shapes of the step kernels (wdem_set_launch_shape) and the autotuner (wdem_autotune).

Results must not depend on the shape: every contact and particle is computed alone and every sum runs
in a fixed order, so each shape gives the default shape's state bit for bit.  The autotuner returns a
valid shape no slower than the one it started from, and the Python engine's autotune option tunes on a
copy of the state, so that a tuned run equals an untuned one bit for bit."""
import numpy as np
import pytest

from woo_gb300 import abi, dem, scenes, utils
from woo_gb300.core import Scene

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu

SHAPES = [dict(contactsBlock=64, contactsPerSM=8, cullBlock=128, integratorBlock=128, listsPerSM=1),
          dict(contactsBlock=256, contactsPerSM=1, cullBlock=512, integratorBlock=512, listsPerSM=2),
          dict(contactsBlock=128, contactsPerSM=16, cullBlock=256, integratorBlock=256, listsPerSM=4)]


@pytest.mark.parametrize("law", ["frict", "hertz"])
def test_shapes_do_not_change_results(wdem_lib, law):
    spec = scenes.random_cloud(3000, 8, box=(0.2, 0.2, 0.2), dense=0.85, law=law)
    ref = gpu_handle(spec)
    ref.step(80)
    pr, cr = gpu_particles(ref, spec.particles.n), ref.download_contacts()
    for shape in SHAPES:
        h = gpu_handle(spec)
        h.set_launch_shape(**shape)
        assert h.launch_shape() == shape
        h.step(80)
        assert_same_particles(gpu_particles(h, spec.particles.n), pr)
        assert_same_contacts(h.download_contacts(), cr)
        h.close()


def test_invalid_shape_rejected(wdem_lib):
    spec = scenes.random_cloud(100, 1)
    h = gpu_handle(spec)
    with pytest.raises(abi.WdemError):
        h.set_launch_shape(contactsBlock=96)
    with pytest.raises(abi.WdemError):
        h.set_launch_shape(cullBlock=1024)


def test_autotune_picks_a_valid_shape(wdem_lib):
    spec = scenes.random_cloud(20000, 4, box=(0.3, 0.3, 0.3), dense=0.85)
    h = gpu_handle(spec)
    h.step(20)
    r = h.autotune(3)
    s = r["shape"]
    assert s["contactsBlock"] in (64, 128, 256) and s["cullBlock"] in (128, 256, 512)
    assert s["integratorBlock"] in (128, 256, 512)
    assert 0 < r["ms"] <= r["ms_start"]
    assert h.launch_shape() == s
    h.step(10)


def test_engine_autotune_does_not_advance_the_run(wdem_lib, tmp_path, monkeypatch):
    monkeypatch.setenv("WOO_GB300_TUNING", str(tmp_path / "shapes.json"))

    def build(autotune):
        m = utils.defaultMaterial()
        S = Scene(dtSafety=0.5, engines=dem.DemField.minimalEngines(damping=0.3, dynDtPeriod=0),
                  fields=[dem.DemField(gravity=(0, 0, -10), par=[dem.Wall.make(0, axis=2, sense=1, mat=m)])])
        rng = np.random.default_rng(2)
        for k in range(400):
            S.dem.par.add(dem.Sphere.make(rng.uniform(0, 0.2, 3) + (0, 0, 0.05), radius=0.004, mat=m))
        S.engines = [dem.GpuDemEngine.fromEngines(S.engines)] + [e for e in S.engines if isinstance(e, dem.DynDt)]
        S.engines[0].autotune = autotune
        return S

    a, b = build(False), build(True)
    a.run(200, True)
    b.run(200, True)
    assert b.engines[0]._tuned is not None
    for pa, pb in zip(a.dem.par, b.dem.par):
        assert tuple(pa.pos) == tuple(pb.pos) and tuple(pa.vel) == tuple(pb.vel)
