"""CPU restatement of the bucket-width controller network and its training
step (float64 numpy), used as the checker of the library's CUDA forward,
backward and Adam kernels (graphbench_gb300/csrc/gbs_mlp.cu).

TEST INFRASTRUCTURE ONLY: imported by tests/ to check gradients; never used
by the product path.

Network: x (16 raw inputs) -> standardise with the block's means / scales ->
W1 (16x64) + b1, ReLU -> W2 (64x64) + b2, ReLU -> W3 (64x2) + b3 -> (y0, y1).
Loss over samples with weights w:
    L = sum_i w_i [ (y0_i - t0_i)^2 + BCE(sigmoid(y1_i), t1_i) ] / sum_i w_i
Parameter block layout (float32, 5410 values): mu[16], sd[16], W1[16][64],
b1[64], W2[64][64], b2[64], W3[64][2], b3[2]; the gradient vector covers the
5378 values after mu and sd, in the same order.
"""
from __future__ import annotations

import numpy as np

F, H = 16, 64
OFF_W1 = 2 * F
OFF_B1 = OFF_W1 + F * H
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * 2
N_FLOATS = OFF_B3 + 2


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[:F], p[F:2 * F], p[OFF_W1:OFF_B1].reshape(F, H), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H),
            p[OFF_B2:OFF_W3], p[OFF_W3:OFF_B3].reshape(H, 2), p[OFF_B3:N_FLOATS])


def forward(p, x):
    mu, sd, W1, b1, W2, b2, W3, b3 = unpack(p)
    xn = (np.asarray(x, dtype=np.float64) - mu) / sd
    h1 = np.maximum(xn @ W1 + b1, 0.0)
    h2 = np.maximum(h1 @ W2 + b2, 0.0)
    y = h2 @ W3 + b3
    return y, (xn, h1, h2)


def loss_grad(p, x, t, w=None):
    """Mean weighted loss and its gradient (5378 values) at parameters p."""
    x = np.asarray(x, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    w = np.ones(len(x)) if w is None else np.asarray(w, dtype=np.float64)
    mu, sd, W1, b1, W2, b2, W3, b3 = unpack(p)
    y, (xn, h1, h2) = forward(p, x)
    ws = w / w.sum()
    e = y[:, 0] - t[:, 0]
    z = y[:, 1]
    bce = np.maximum(z, 0) - z * t[:, 1] + np.log1p(np.exp(-np.abs(z)))
    loss = float(np.sum(ws * (e * e + bce)))
    dy = np.stack([2 * e * ws, (1 / (1 + np.exp(-z)) - t[:, 1]) * ws], axis=1)
    gW3 = h2.T @ dy
    gb3 = dy.sum(0)
    dh2 = (dy @ W3.T) * (h2 > 0)
    gW2 = h1.T @ dh2
    gb2 = dh2.sum(0)
    dh1 = (dh2 @ W2.T) * (h1 > 0)
    gW1 = xn.T @ dh1
    gb1 = dh1.sum(0)
    g = np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
    return loss, g


def adam(p, g, m, v, step, lr, beta1=0.9, beta2=0.999, eps=1e-8):
    """One bias-corrected Adam step on the trained part of p (returns new p, m, v)."""
    p = np.asarray(p, dtype=np.float64).copy()
    m = beta1 * m + (1 - beta1) * g
    v = beta2 * v + (1 - beta2) * g * g
    mh = m / (1 - beta1 ** step)
    vh = v / (1 - beta2 ** step)
    p[OFF_W1:] -= lr * mh / (np.sqrt(vh) + eps)
    return p, m, v


def init_params(seed: int, mu=None, sd=None):
    """He-initialised block with the given standardisation."""
    rng = np.random.default_rng(seed)
    p = np.zeros(N_FLOATS, dtype=np.float64)
    p[:F] = 0.0 if mu is None else mu
    p[F:2 * F] = 1.0 if sd is None else sd
    p[OFF_W1:OFF_B1] = rng.normal(0, np.sqrt(2 / F), F * H)
    p[OFF_W2:OFF_B2] = rng.normal(0, np.sqrt(2 / H), H * H)
    p[OFF_W3:OFF_B3] = rng.normal(0, np.sqrt(1 / H), H * 2)
    return p.astype(np.float32)
