"""The CPU reference of the warm-start network: its backward pass against finite differences (in
float64), and the BF16 rounding helper against its definition."""
import numpy as np

from oracle import warm_mlp as M


def test_bf16_rounding():
    x = np.array([1.0, 1.0 + 2 ** -7, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -8, -2.5, 0.0, 3.0e-5], np.float32)
    r = M.bf16(x)
    # 7 fraction bits: 1 + 2^-7 is representable; 1 + 2^-8 is a tie -> even (1.0);
    # 1 + 3 * 2^-8 is a tie between 1 + 2^-7 (odd) and 1 + 2^-6 (even) -> 1 + 2^-6
    assert r[0] == 1.0 and r[1] == np.float32(1.0 + 2 ** -7) and r[2] == 1.0 and r[3] == np.float32(1.0 + 2 ** -6)
    assert r[4] == -2.5 and r[5] == 0.0
    assert abs(r[6] - 3.0e-5) <= 3.0e-5 * 2 ** -8


def test_backward_matches_finite_differences():
    rng = np.random.default_rng(0)
    w = M.init(1) * 0.5 + rng.normal(0, 0.01, M.NPARAM)
    R = rng.normal(0, 0.5, (40, 17))
    loss, g = M.loss_grad(w, R, bf=False)
    idx = rng.choice(M.NPARAM, 60, replace=False)
    eps = 1e-6
    for k in idx:
        wp, wm = w.copy(), w.copy()
        wp[k] += eps
        wm[k] -= eps
        fd = (M.loss_grad(wp, R, bf=False)[0] - M.loss_grad(wm, R, bf=False)[0]) / (2 * eps)
        assert abs(fd - g[k]) <= 1e-6 * max(1.0, abs(fd)), (k, fd, g[k])
