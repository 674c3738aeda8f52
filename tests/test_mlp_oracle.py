"""CPU: the network oracle's backward pass agrees with central finite differences (FP64)."""
from __future__ import annotations

import numpy as np

import mlp_oracle as M


def test_oracle_gradient_matches_finite_differences():
    rng = np.random.default_rng(0)
    p = M.init_params(rng)
    p[M.B1:M.W2] = rng.standard_normal(64) * 0.1
    p[M.B2:M.W3] = rng.standard_normal(64) * 0.1
    p[M.B3] = 0.05
    n = 40
    x0 = rng.uniform(-2, 0.5, n)
    x1 = rng.uniform(0, 1, n)
    y = rng.uniform(0, 0.3, n)
    w = (rng.uniform(size=n) > 0.3).astype(float)
    _, g = M.loss_and_grad(p, x0, x1, y, w)
    idx = np.concatenate([np.arange(0, 128, 9), np.arange(128, 192, 7), rng.choice(np.arange(192, 4288), 40, replace=False),
                          np.arange(4288, 4352, 5), np.arange(4352, 4416, 6), [4416]])
    h = 1e-6
    for i in idx:
        pp, pm = p.copy(), p.copy()
        pp[i] += h
        pm[i] -= h
        fd = (M.loss_and_grad(pp, x0, x1, y, w)[0] - M.loss_and_grad(pm, x0, x1, y, w)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])), (i, fd, g[i])


def test_bf16_rounding_is_round_to_nearest_even():
    vals = np.array([1.0, 1.00390625, 1.0078125, 1.005859375, -3.14159, 65504.0, 1e-20], dtype=np.float32)
    r = M.bf16(vals)
    for v, b in zip(vals, r):
        # the result is representable in 8 significand bits and within half an ulp
        assert abs(b - v) <= abs(v) * 2.0 ** -8 + 1e-45
    assert M.bf16(np.float32(1.005859375)) == 1.0078125  # tie -> even


def test_forward_matches_loss_path():
    rng = np.random.default_rng(1)
    p = M.init_params(rng)
    x0, x1 = rng.uniform(-2, 0, 16), rng.uniform(0, 1, 16)
    f = M.forward(p, x0, x1)
    loss, _ = M.loss_and_grad(p, x0, x1, f, np.ones(16))
    assert loss < 1e-24
