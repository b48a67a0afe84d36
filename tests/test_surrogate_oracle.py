"""CPU checks of the surrogate's float64 restatement (oracle/surrogate_mlp.py):
its backward pass against central finite differences, and the bfloat16
rounding it uses to emulate the tensor-core path."""
import numpy as np

import surrogate_mlp as M


def _norm(seed=1):
    rng = np.random.default_rng(seed)
    lo = np.array([0.0, -0.1, -0.1, 0.4])
    sc = 2.0 / np.array([1.5, 0.2, 0.2, 0.6])
    freq = np.pi * rng.normal(0, [3.0, 1.0, 1.0, 0.5], size=(M.FREQ, 4))
    mean = rng.normal(0, 1, M.OUT)
    std = rng.uniform(0.5, 2.0, M.OUT)
    return np.concatenate([lo, sc, freq.ravel(), mean, std]).astype(np.float32)


def _batch(n, seed=2):
    rng = np.random.default_rng(seed)
    x = np.stack([rng.uniform(0, 1.5, n), rng.uniform(-0.1, 0.1, n), rng.uniform(-0.1, 0.1, n),
                  rng.uniform(0.4, 1.0, n)], axis=1).astype(np.float32)
    t = rng.normal(0, 1, (n, M.OUT)).astype(np.float32)
    return x, t


def test_backward_matches_finite_differences():
    params = M.random_params(3).astype(np.float64)
    norm = _norm()
    x, t = _batch(16)
    _, g = M.loss_grad(params, norm, x, t)
    rng = np.random.default_rng(4)
    # a sample of parameters from every block: weights and biases of each layer
    idx = []
    for l in range(M.HIDDEN):
        idx += list(l * M.LAYER + rng.integers(0, M.WIDTH * M.WIDTH, 6))
        idx += list(l * M.LAYER + M.WIDTH * M.WIDTH + rng.integers(0, M.WIDTH, 3))
    idx += list(M.W5 + rng.integers(0, M.OUT * M.WIDTH, 6)) + list(M.B5 + np.arange(M.OUT))
    h = 1e-6
    for i in idx:
        p1, p0 = params.copy(), params.copy()
        p1[i] += h
        p0[i] -= h
        fd = (M.loss_grad(p1, norm, x, t)[0] - M.loss_grad(p0, norm, x, t)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-8, (i, fd, g[i])
    # padded output rows receive no gradient
    assert np.all(g[M.W5 + M.OUT * M.WIDTH:M.B5] == 0) and np.all(g[M.B5 + M.OUT:] == 0)


def test_bf16_rounding():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, -2.5, 1e-3, 3.0e38], dtype=np.float32)
    r = M.bf16(v)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: rounds to even (1); 1 + 3*2^-9 rounds up
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0 + 2 ** -7 and r[3] == -2.5
    assert abs(r[4] - 1e-3) <= 1e-3 * 2 ** -8
    assert np.all(r.astype(np.float32).view(np.uint32) & 0xFFFF == 0)
