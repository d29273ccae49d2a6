"""DynDt on the GPU against the oracle: the critical step from the contact stiffnesses, the new dt
(bitwise) and the state that follows from it, under the PeriodicEngine schedule; and through the
Woo-style surface (defaultEngines with DynDt)."""
import numpy as np
import pytest

from oracle import bridge
from woo_gb300 import abi, dem, scenes, utils
from woo_gb300.core import Scene

from helpers import assert_same_contacts, assert_same_particles, gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("law", ["frict", "hertz"])
@pytest.mark.parametrize("period", [1, 7])
def test_dyndt_bitexact(wdem_lib, law, period):
    spec = scenes.random_cloud(400, 4, dense=0.85, law=law)
    spec.params.dynDtPeriod = period
    spec.params.dynDtMaxRelInc = 1e-3
    spec.params.dtSafety = 0.6
    spec.params.dt = spec.params.dt * 0.5
    n = spec.particles.n
    h = gpu_handle(spec)
    o = bridge.Oracle(spec.params, spec.particles)
    changed = 0
    last = spec.params.dt
    for chunk in (1, 6, 30, 113):
        h.step(chunk)
        o.step(chunk)
        st = h.status()
        assert st.dt == o.dt(), f"dt {st.dt!r} != {o.dt()!r}"
        assert (np.isnan(st.dynDtCrit) and np.isnan(o.dyndt_crit())) or st.dynDtCrit == o.dyndt_crit()
        changed += st.dt != last
        last = st.dt
        assert_same_particles(gpu_particles(h, n), o.particles())
        assert_same_contacts(h.download_contacts(), o.contacts())
    assert changed > 0, "dt never changed"


def test_dyndt_woo_surface(wdem_lib):
    m = dem.FrictMat(young=1e7, density=2000)
    par = [dem.Wall.make(0, axis=2, sense=1, mat=m)]
    rng = np.random.default_rng(1)
    for k in range(60):
        par.append(dem.Sphere.make((0.03 * (k % 6), 0.03 * ((k // 6) % 5), 0.012 + 0.025 * (k // 30)), 0.012, mat=m))
    S = Scene(fields=[dem.DemField(gravity=(0, 0, -9.81), par=par)],
              engines=utils.defaultEngines(damping=0.3, dynDtPeriod=10), dtSafety=0.5)
    S.run(1)
    dt0 = S.dt
    t = S.time
    S.run(300)
    assert S.step == 301
    assert S.dt != dt0
    assert S.time > t
    assert S._engine()._h.status().dynDtCrit > 0
