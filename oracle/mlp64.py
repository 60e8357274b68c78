"""Float64 NumPy surrogate MLP: forward, backward and Adam (test infrastructure).

The reference has no learned model; this is the project's own CPU restatement of
the network the device kernels train (csrc/mlp.cu): layers l = 0..3 with
z_l = a_l W_l^T + b_l, a_{l+1} = silu(z_l) for l < 3, y = z_3, loss
mean((y - t)^2) over batch and outputs, and bias-corrected Adam.  Parameters use
the device's flat per-member layout (pc_mlp_param_layout): for each layer the
weight [n][k] (k of layer 0 padded to 32 with zero columns) then the bias [n].
It is cross-checked against torch float64 autograd in the CPU tests and is the
checker of the device gradients in the GPU tests; nothing in the product path
imports it.
"""

from __future__ import annotations

import numpy as np


def layout(dims):
    """[(w_off, b_off, n, k)] per layer and the per-member parameter count."""
    segs, off = [], 0
    for l in range(4):
        k = 32 if l == 0 else dims[l]
        n = dims[l + 1]
        segs.append((off, off + n * k, n, k))
        off += n * k + n
    return segs, off


def unpack(p, dims):
    segs, _ = layout(dims)
    Ws, bs = [], []
    for w_off, b_off, n, k in segs:
        Ws.append(p[w_off:w_off + n * k].reshape(n, k))
        bs.append(p[b_off:b_off + n])
    return Ws, bs


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def forward(p, x, dims):
    """x [B][dims[0]] -> (y [B][dims[4]], cache)."""
    Ws, bs = unpack(np.asarray(p, dtype=np.float64), dims)
    a = np.zeros((x.shape[0], 32))
    a[:, : x.shape[1]] = x
    acts, zs = [a], []
    for l in range(4):
        z = acts[-1] @ Ws[l].T + bs[l]
        zs.append(z)
        if l < 3:
            acts.append(silu(z))
    return zs[-1], (acts, zs, Ws)


def loss_and_grads(p, x, t, dims):
    """Mean-squared error and its gradient in the flat parameter layout."""
    y, (acts, zs, Ws) = forward(p, x, dims)
    B, N = y.shape
    d = y - t
    loss = float(np.mean(d * d))
    g = 2.0 * d / (B * N)
    segs, P = layout(dims)
    grad = np.zeros(P)
    for l in range(3, -1, -1):
        w_off, b_off, n, k = segs[l]
        grad[w_off:w_off + n * k] = (g.T @ acts[l]).ravel()
        grad[b_off:b_off + n] = g.sum(axis=0)
        if l > 0:
            g = (g @ Ws[l]) * dsilu(zs[l - 1])
    return loss, grad


def adam_step(p, grad, m, v, t, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One bias-corrected Adam step (t counts from 1); returns new (p, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    lr_t = lr * np.sqrt(1 - b2**t) / (1 - b1**t)
    return p - lr_t * m / (np.sqrt(v) + eps), m, v


def init_params(dims, rng):
    """Uniform(+-sqrt(6 / (fan_in + fan_out))) weights, zero biases, zero padding."""
    segs, P = layout(dims)
    p = np.zeros(P)
    for l, (w_off, b_off, n, k) in enumerate(segs):
        fan_in = dims[l]
        lim = np.sqrt(6.0 / (fan_in + n))
        w = np.zeros((n, k))
        w[:, :fan_in] = rng.uniform(-lim, lim, size=(n, fan_in))
        p[w_off:w_off + n * k] = w.ravel()
    return p
