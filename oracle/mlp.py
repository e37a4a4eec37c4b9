"""Test infrastructure: numpy FP64 oracle of the surrogate MLP (forward, MSE loss, backward, Adam).

The network is n_in -> H -> H -> n_out with tanh hidden layers and a linear output; loss is
the mean of squared errors over all outputs. With bf16=True the operands are rounded to BF16
at the points where the GPU kernels round them (inputs, weights, hidden biases, hidden
pre-activations and activations, the output gradient and the back-propagated pre-activation
gradients), so the GPU gradients can
be compared tightly; with bf16=False it is plain FP64 (what the finite-difference check uses).
Only tests import this module.
"""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(x, np.float32)
    b = f.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def _r(x, on):
    return bf16(x) if on else np.asarray(x, np.float64)


def forward(params, X, bf16_ops=True):
    W1, b1, W2, b2, W3, b3 = [np.asarray(p, np.float64) for p in params]
    r = lambda x: _r(x, bf16_ops)  # noqa: E731
    Xr = r(X)
    # the GPU rounds the pre-activation to BF16 pairs and takes tanh in BF16 (tanh.approx.bf16x2);
    # the hidden biases enter in BF16 (the inference kernel adds them on the tensor core)
    H1 = r(np.tanh(r(Xr @ r(W1).T + r(b1))))
    H2 = r(np.tanh(r(H1 @ r(W2).T + r(b2))))
    Y = H2 @ r(W3).T + b3
    return Y, (Xr, H1, H2)


def loss_grad(params, X, T, bf16_ops=True):
    """Mean squared error and gradients (same order as params)."""
    W1, b1, W2, b2, W3, b3 = [np.asarray(p, np.float64) for p in params]
    r = lambda x: _r(x, bf16_ops)  # noqa: E731
    Y, (Xr, H1, H2) = forward(params, X, bf16_ops)
    n, m = Y.shape
    D = Y - np.asarray(T, np.float64)
    loss = float((D ** 2).mean())
    dY = r(2.0 * D / (n * m))
    dZ2 = r((dY @ r(W3)) * (1.0 - H2 ** 2))
    dZ1 = r((dZ2 @ r(W2)) * (1.0 - H1 ** 2))
    grads = [dZ1.T @ Xr, dZ1.sum(0), dZ2.T @ H1, dZ2.sum(0), dY.T @ H2, dY.sum(0)]
    return loss, grads


def adam(params, grads, m, v, step, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step (Kingma & Ba 2015) in FP64; returns new params, m, v."""
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    out_p, out_m, out_v = [], [], []
    for p, g, mi, vi in zip(params, grads, m, v):
        mi = b1 * mi + (1 - b1) * g
        vi = b2 * vi + (1 - b2) * g * g
        out_p.append(p - lr * (mi / c1) / (np.sqrt(vi / c2) + eps))
        out_m.append(mi)
        out_v.append(vi)
    return out_p, out_m, out_v
