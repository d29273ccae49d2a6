"""The learned warm start on the GPU: tensor-core forward and backward against the CPU reference of
the network (oracle/warm_mlp.py, same BF16 rounding points), Adam training on records logged by the
plain Newton solver, and what the trained network gains over the cold start."""
import numpy as np
import pytest

from oracle import warm_mlp as M
from woo_gb300 import abi, scenes

from helpers import gpu_handle, gpu_particles

pytestmark = pytest.mark.gpu


def _features(rng, n):
    """Feature rows in the ranges the solver produces: offset in [-1, 1], unit quaternion with w >= 0,
    semi-axes in (0, 0.5]."""
    X = np.zeros((n, 13), np.float32)
    X[:, :3] = rng.uniform(-1, 1, (n, 3))
    q = rng.normal(size=(n, 4))
    q /= np.linalg.norm(q, axis=1)[:, None]
    q[q[:, 0] < 0] *= -1
    X[:, 3:7] = q
    X[:, 7:13] = rng.uniform(0.1, 0.5, (n, 6))
    return X


def _handle():
    spec = scenes.ellipsoid_cloud(20, 1)
    return gpu_handle(spec)


def test_forward_matches_reference(wdem_lib):
    h = _handle()
    h.warm_init(3)
    w = h.warm_get_weights().astype(np.float64)
    X = _features(np.random.default_rng(0), 1000)
    Yg = h.warm_predict(X)
    Yr, _ = M.forward(w, X)
    # the tcgen05 kernel accumulates in FP32 like the reference's float64 sums rounded at the same BF16
    # points; a BF16 re-rounding of an activation that lands on a rounding boundary could move an output by
    # one BF16 ulp of that activation's contribution, which the 1e-3 bound would still cover
    assert np.abs(Yg - Yr).max() <= 1e-3 * np.abs(Yr).max()
    assert np.corrcoef(Yg.ravel(), Yr.ravel())[0, 1] > 0.999999


def test_gradient_matches_reference(wdem_lib):
    h = _handle()
    h.warm_init(5)
    w = h.warm_get_weights().astype(np.float64)
    rng = np.random.default_rng(1)
    R = np.zeros((300, 17), np.float32)
    R[:, :13] = _features(rng, 300)
    R[:, 13] = rng.uniform(0.2, 0.8, 300)
    R[:, 14:] = rng.uniform(-0.5, 0.5, (300, 3))
    g, loss = h.warm_grad(R)
    lr, gr = M.loss_grad(w, R.astype(np.float64))
    assert loss == pytest.approx(lr, rel=5e-3)
    # layer by layer: relative error of the gradient block
    q = 0
    for fi, fo in ((13, 64), (64, 64), (64, 64), (64, 4)):
        for size in (fi * fo, fo):
            a, b = g[q:q + size], gr[q:q + size]
            q += size
            assert np.linalg.norm(a - b) <= 3e-2 * np.linalg.norm(b) + 1e-9, (fi, fo, size)


def _iters(spec, weights=None):
    h = gpu_handle(spec)
    if weights is not None:
        h.warm_set_weights(weights)
    h.step(40)
    st = h.status()
    return h, st.ellIters / st.ellSolves, st.ellFallbacks / st.ellSolves


def test_training_gain(wdem_lib):
    """Records logged by the plain (cold-start) Newton solver on one packing train the network; on
    another packing its warm start needs fewer Newton iterations per solve than the cold start, at the
    same 1e-10 tolerance and with the same trajectory."""
    src = scenes.ellipsoid_cloud(12000, 11, box=(0.3, 0.3, 0.3), dense=0.75, ellSolver=abi.ELL_NEWTON,
                                 warmStart=abi.WARM_COLD)
    h = gpu_handle(src)
    h.ell_log(2_000_000)
    h.step(100)
    R = h.ell_log_read(2_000_000)
    assert len(R) > 300_000
    assert np.all((R[:, 13] > 0) & (R[:, 13] < 1))
    losses = h.warm_train(R, epochs=12, batch=512, lr=3e-3, seed=1)
    assert losses[-1] < 0.5 * losses[0]
    w = h.warm_get_weights()

    cold = scenes.ellipsoid_cloud(1500, 12, dense=0.75, ellSolver=abi.ELL_NEWTON, warmStart=abi.WARM_COLD)
    mlp = scenes.ellipsoid_cloud(1500, 12, dense=0.75, ellSolver=abi.ELL_NEWTON, warmStart=abi.WARM_MLP)
    hc, ic, _ = _iters(cold)
    hm, im, fb = _iters(mlp, w)
    print(f"warm-start gain: {len(R)} records, loss {losses[0]:.3e} -> {losses[-1]:.3e}; Newton iterations per "
          f"solve cold {ic:.3f}, learned {im:.3f}, fallbacks {fb:.4f}")
    assert im < 0.85 * ic, (im, ic)
    assert fb < 0.05
    pc, pm = gpu_particles(hc, cold.particles.n), gpu_particles(hm, mlp.particles.n)
    assert np.allclose(pc.pos, pm.pos, rtol=0, atol=1e-9 * np.abs(pc.pos).max())
    # the previous step's lambda where a pair has one, the network for pairs solved for the first time:
    # fewer iterations than the history warm start alone on the same run, the same trajectory
    hist = scenes.ellipsoid_cloud(1500, 12, dense=0.75, ellSolver=abi.ELL_NEWTON, warmStart=abi.WARM_HISTORY)
    both = scenes.ellipsoid_cloud(1500, 12, dense=0.75, ellSolver=abi.ELL_NEWTON, warmStart=abi.WARM_HISTORY_MLP)
    hh, ih, _ = _iters(hist)
    hb, ib, fbb = _iters(both, w)
    print(f"history {ih:.3f}, history + learned {ib:.3f} Newton iterations per solve (fallbacks {fbb:.4f})")
    assert ib <= ih and ib < ic
    pb = gpu_particles(hb, both.particles.n)
    assert np.allclose(pc.pos, pb.pos, rtol=0, atol=1e-9 * np.abs(pc.pos).max())



def test_forward_large_batch(wdem_lib):
    """2^20 rows through the tensor-core kernel (8192 tiles of 128 over the persistent CTAs): a seeded
    sample of 4096 rows against the reference, every output finite."""
    h = _handle()
    h.warm_init(3)
    w = h.warm_get_weights().astype(np.float64)
    rng = np.random.default_rng(7)
    X = _features(rng, 1 << 20)
    Yg = h.warm_predict(X)
    assert np.isfinite(Yg).all()
    pick = rng.choice(len(X), 4096, replace=False)
    Yr, _ = M.forward(w, X[pick])
    assert np.abs(Yg[pick] - Yr).max() <= 1e-3 * np.abs(Yr).max()
