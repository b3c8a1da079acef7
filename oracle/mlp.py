"""CPU oracle of the surrogate network (test infrastructure only).

A float64 numpy restatement of the BF16 multilayer perceptron that
create_rate_subs_gb300.surrogate trains on the GPU: forward pass, mean
squared error, the backward pass and one Adam update.  With ``bf16=True``
values are rounded to bfloat16 at exactly the points where the GPU kernels
store them in bf16 (the network input, the hidden activations, the output
gradient and the hidden-layer gradients), so the only remaining difference
is the accumulation precision (float64 here, fp32 on the tensor cores).

The reference has no network; this oracle pins the kernels' gradients, the
way the reference's emitted C pins the rate kernels.
"""
import numpy as np

__all__ = ["bf16_round", "silu", "dsilu", "forward", "loss_and_grads", "adam"]


def bf16_round(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(X, Ws, bs, bf16=True):
    """Network output and the per-layer (input, pre-activation) pairs.

    X: (m, n_in); Ws[l]: (n_out, n_in); bs[l]: (n_out,).  Hidden layers use
    SiLU, the last layer is linear."""
    r = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    a = r(X)
    cache = []
    L = len(Ws)
    for l in range(L):
        z = a @ r(Ws[l]).T + bs[l]
        cache.append((a, z))
        a = r(silu(z)) if l < L - 1 else z
    return a, cache


def loss_and_grads(X, Tg, Ws, bs, bf16=True):
    """MSE loss (mean over all m * n_out entries) and its gradients."""
    r = bf16_round if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    Yh, cache = forward(X, Ws, bs, bf16)
    m, n = Tg.shape
    scale = 1.0 / (m * n)
    d = Yh - Tg
    loss = float(np.sum(d * d) * scale)
    dz = r(2.0 * scale * d)
    gW = [None] * len(Ws)
    gb = [None] * len(Ws)
    for l in range(len(Ws) - 1, -1, -1):
        a, _ = cache[l]
        gW[l] = dz.T @ a
        gb[l] = dz.sum(axis=0)
        if l > 0:
            z_prev = cache[l - 1][1]
            dz = r((dz @ r(Ws[l])) * dsilu(z_prev))
    return loss, gW, gb


def adam(p, g, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step; returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    c1 = 1.0 / (1.0 - b1 ** step)
    c2 = 1.0 / (1.0 - b2 ** step)
    return p - lr * (m * c1) / (np.sqrt(v * c2) + eps), m, v
