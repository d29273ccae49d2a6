"""CPU reference of the learned warm start network (TEST INFRASTRUCTURE ONLY).

Restates, in numpy, the forward and backward pass of the 13 -> 64 -> 64 -> 64 -> 4 ReLU network that
the GPU engine runs on its tensor cores (woo_gb300/csrc/k_mlp.cu), with the same rounding points:
inputs, weights and post-ReLU activations rounded to BF16 (round to nearest even), the dZ operands of
the backward products rounded to BF16, accumulation in higher precision (the GPU accumulates in FP32),
biases, pre-activations and outputs unrounded.  With bf16=False the same code runs in float64 and is
checked against finite differences.  The network is new (it has no counterpart in the reference); its
targets are the Perram-Wertheim maximiser of Cg2_Ellipsoid_Ellipsoid_L6Geom (Ellipsoid.cpp:270-351).
"""
import numpy as np

NIN, H, NOUT = 13, 64, 4
NPARAM = NIN * H + H + H * H + H + H * H + H + H * NOUT + NOUT
LOSS_W = np.array([1.0, 0.1, 0.1, 0.1])


def bf16(x):
    """Round float32 values to the nearest BF16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(np.asarray(x, np.float32))
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000).astype(np.uint32)
    return r.view(np.float32).reshape(a.shape)


def unpack(w):
    """Public parameter vector -> [(W1, b1), (W2, b2), (W3, b3), (W4, b4)], W[l] of shape (in, out)."""
    w = np.asarray(w, np.float64)
    out, q = [], 0
    for fi, fo in ((NIN, H), (H, H), (H, H), (H, NOUT)):
        W = w[q:q + fi * fo].reshape(fi, fo); q += fi * fo
        b = w[q:q + fo]; q += fo
        out.append((W, b))
    assert q == NPARAM
    return out


def pack(layers):
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in layers])


def forward(w, X, bf=True):
    """Outputs (n, 4) and the activations needed by backward."""
    rnd = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    L = unpack(w)
    a = rnd(X).astype(np.float64)
    acts = [a]
    for li, (W, b) in enumerate(L):
        z = a @ rnd(W).astype(np.float64) + b
        if li < 3:
            a = rnd(np.maximum(z, 0.0)).astype(np.float64)
            acts.append(a)
        else:
            out = z
    return out, acts


def loss_grad(w, R, bf=True):
    """Mean weighted squared error over records R (n, 17) and its gradient (public layout)."""
    rnd = bf16 if bf else (lambda v: np.asarray(v, np.float64))
    n = len(R)
    X, Y = R[:, :NIN], R[:, NIN:NIN + NOUT]
    out, acts = forward(w, X, bf)
    e = out - Y
    loss = float(np.sum(LOSS_W * e * e) / n)
    dz = 2.0 * LOSS_W * e / n
    L = unpack(w)
    grads = [None] * 4
    dzr = rnd(dz).astype(np.float64)
    for li in range(3, -1, -1):
        W, _ = L[li]
        gb = dz.sum(axis=0)
        gW = acts[li].T @ dzr
        grads[li] = (gW, gb)
        if li > 0:
            da = dzr @ rnd(W).astype(np.float64).T
            dz = da * (acts[li] > 0)
            dzr = rnd(dz).astype(np.float64)
    return loss, pack(grads)


def init(seed):
    """He-uniform weights and zero biases, the same construction as wdem_warm_init (not the same
    random numbers)."""
    rng = np.random.default_rng(seed)
    layers = []
    for fi, fo in ((NIN, H), (H, H), (H, H), (H, NOUT)):
        lim = np.sqrt(6.0 / fi)
        layers.append((rng.uniform(-lim, lim, (fi, fo)), np.zeros(fo)))
    return pack(layers)
