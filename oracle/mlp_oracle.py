"""FP64 CPU restatement of the learned field model (no reference counterpart):
Fourier features, MLP forward, MSE loss and backward.

TEST INFRASTRUCTURE ONLY: the checker of the GPU training kernels' gradients.
Layer sizes 128 -> 256 -> 256 -> 256 -> 256 -> 6 with SiLU; parameters in one
flat array W0, b0, ..., W4, b4 with W_l stored [out][in].
"""
import numpy as np

SIZES = [(128, 256), (256, 256), (256, 256), (256, 256), (256, 6)]


def unflatten(p):
    out, off = [], 0
    for i, o in SIZES:
        w = p[off:off + i * o].reshape(o, i)
        off += i * o
        b = p[off:off + o]
        off += o
        out.append((w, b))
    return out


def features(u32, freq):
    """u32: n x 3 box fractions in 32-bit fixed point; freq: 64 x 3 integers.
    Phase n.u mod 1 formed exactly in integers, as the device does."""
    u = np.asarray(u32, dtype=np.uint64)
    f = np.asarray(freq, dtype=np.int64).astype(np.uint64)
    ph = (u @ f.T) & np.uint64(0xFFFFFFFF)          # n x 64, mod 2^32
    rev = ph.astype(np.int64)
    rev = np.where(rev >= 2 ** 31, rev - 2 ** 32, rev).astype(np.float64) / 2 ** 32
    a = 2 * np.pi * rev
    return np.concatenate([np.sin(a), np.cos(a)], axis=1)


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(params, x):
    zs, hs = [], [x]
    h = x
    for l, (w, b) in enumerate(params):
        z = h @ w.T + b
        if l < len(params) - 1:
            zs.append(z)
            h = silu(z)
            hs.append(h)
        else:
            y = z
    return y, zs, hs


def loss_and_grads(p_flat, x, t_norm):
    """Mean squared error over n x 6 outputs and its gradient (flat layout)."""
    params = unflatten(p_flat)
    y, zs, hs = forward(params, x)
    n = len(x)
    r = y - t_norm
    loss = np.mean(r * r)
    dy = 2.0 * r / (n * 6)
    grads = []
    g = dy
    for l in range(len(params) - 1, -1, -1):
        w, _ = params[l]
        dw = g.T @ hs[l]
        db = g.sum(axis=0)
        grads.append((dw, db))
        if l > 0:
            g = (g @ w) * silu_grad(zs[l - 1])
    grads = grads[::-1]
    flat = np.concatenate([np.concatenate([dw.ravel(), db]) for dw, db in grads])
    return loss, y, flat
