"""Float64 restatement of the learned field surrogate's network (the math of
magrathea-pathfinder_gb300/csrc/mpf_surrogate.cu), for checking its training
gradients and its tensor-core inference.

TEST INFRASTRUCTURE ONLY: the checker for the CUDA path in tests/.  Nothing in
the product imports it.  The surrogate has no counterpart in the reference
(the reference always gathers from the octree), so this file restates the
network's own definition:

  u   = (p - lo) * sc - 1,  p = (x, y, z, a)
  s_j = F_j . u  (j < 64),  h0 = [sin s, cos s]
  h_l = silu(W_l h_(l-1) + b_l)  (l = 1..4, width 128)
  y   = W_5 h_4 + b_5  (16 rows, the first 5 used)
  loss = mean over rows and the 5 outputs of (y - (t - mean) / std)^2
"""
from __future__ import annotations

import numpy as np

WIDTH, HIDDEN, FREQ, OUT, OUT_PAD = 128, 4, 64, 5, 16
LAYER = WIDTH * WIDTH + WIDTH
W5 = HIDDEN * LAYER
B5 = W5 + OUT_PAD * WIDTH
NPARAMS = B5 + OUT_PAD
NNORM = 4 + 4 + FREQ * 4 + OUT + OUT


def unpack_norm(norm):
    norm = np.asarray(norm, dtype=np.float64)
    lo, sc = norm[0:4], norm[4:8]
    freq = norm[8:8 + 4 * FREQ].reshape(FREQ, 4)
    mean = norm[8 + 4 * FREQ:8 + 4 * FREQ + OUT]
    std = norm[8 + 4 * FREQ + OUT:NNORM]
    return lo, sc, freq, mean, std


def unpack_params(params):
    p = np.asarray(params, dtype=np.float64)
    Ws = [p[l * LAYER:l * LAYER + WIDTH * WIDTH].reshape(WIDTH, WIDTH) for l in range(HIDDEN)]
    bs = [p[l * LAYER + WIDTH * WIDTH:(l + 1) * LAYER] for l in range(HIDDEN)]
    Ws.append(p[W5:B5].reshape(OUT_PAD, WIDTH))
    bs.append(p[B5:NPARAMS])
    return Ws, bs


def features(norm, x):
    lo, sc, freq, _, _ = unpack_norm(norm)
    u = (np.asarray(x, dtype=np.float64) - lo) * sc - 1.0
    s = u @ freq.T
    return np.concatenate([np.sin(s), np.cos(s)], axis=1)


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def bf16(a):
    """Round float values to bfloat16 (nearest, ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(params, norm, x, emulate_bf16: bool = False):
    """Normalised outputs (n x 5).  emulate_bf16: the tensor-core path's
    roundings: bfloat16 features and weights, and the activation formed on
    bfloat16 pairs as h + h tanh(h) with h = z / 2 rounded to bfloat16."""
    Ws, bs = unpack_params(params)
    h = features(norm, x)
    if emulate_bf16:
        h = bf16(h)
        Ws = [bf16(W) for W in Ws]
    for l in range(HIDDEN):
        z = h @ Ws[l].T + bs[l]
        if emulate_bf16:
            hh = bf16(0.5 * z)
            h = bf16(hh + hh * bf16(np.tanh(hh)))
        else:
            h = _silu(z)
    y = h @ Ws[HIDDEN].T + bs[HIDDEN]
    return y[:, :OUT]


def field(params, norm, x, emulate_bf16: bool = False):
    """Outputs in field units: phi, dphidx, dphidy, dphidz, dphidt."""
    _, _, _, mean, std = unpack_norm(norm)
    return forward(params, norm, x, emulate_bf16) * std + mean


def loss_grad(params, norm, x, t):
    """Training loss and its gradient with respect to the flat parameters."""
    Ws, bs = unpack_params(params)
    _, _, _, mean, std = unpack_norm(norm)
    tn = (np.asarray(t, dtype=np.float64) - mean) / std
    n = tn.shape[0]
    hs, zs = [features(norm, x)], []
    for l in range(HIDDEN):
        z = hs[-1] @ Ws[l].T + bs[l]
        zs.append(z)
        hs.append(_silu(z))
    y = hs[-1] @ Ws[HIDDEN].T + bs[HIDDEN]
    d = y[:, :OUT] - tn
    loss = float(np.mean(d * d))
    dy = np.zeros((n, OUT_PAD))
    dy[:, :OUT] = 2.0 * d / (n * OUT)
    grad = np.zeros(NPARAMS)
    grad[W5:B5] = (dy.T @ hs[HIDDEN]).ravel()
    grad[B5:NPARAMS] = dy.sum(axis=0)
    dz = (dy @ Ws[HIDDEN]) * _dsilu(zs[HIDDEN - 1])
    for l in range(HIDDEN - 1, -1, -1):
        grad[l * LAYER:l * LAYER + WIDTH * WIDTH] = (dz.T @ hs[l]).ravel()
        grad[l * LAYER + WIDTH * WIDTH:(l + 1) * LAYER] = dz.sum(axis=0)
        if l > 0:
            dz = (dz @ Ws[l]) * _dsilu(zs[l - 1])
    return loss, grad


def random_params(seed: int = 0, scale: float = 1.0):
    """LeCun-normal weights and small random biases (rows 5..15 of the output layer zero)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAMS)
    for l in range(HIDDEN):
        p[l * LAYER:l * LAYER + WIDTH * WIDTH] = rng.normal(0, scale / np.sqrt(WIDTH), WIDTH * WIDTH)
        p[l * LAYER + WIDTH * WIDTH:(l + 1) * LAYER] = rng.normal(0, 0.1, WIDTH)
    p[W5:W5 + OUT * WIDTH] = rng.normal(0, 1 / np.sqrt(WIDTH), OUT * WIDTH)
    p[B5:B5 + OUT] = rng.normal(0, 0.1, OUT)
    return p.astype(np.float32)
