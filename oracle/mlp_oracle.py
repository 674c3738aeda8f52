"""CPU oracle for the continuation-value network of the learned LSM regression.

TEST INFRASTRUCTURE ONLY: the checker for the GPU training and inference
kernels (derivative-pricing_gb300/csrc/lsm_mlp.cu), never part of the product.

Network: x = (x0, x1) -> z1 = W1 x + b1 -> h1 = gelu(z1) -> z2 = W2 h1 + b2 ->
h2 = gelu(z2) -> f = W3 . h2 + b3, with gelu the tanh form
gelu(z) = z/2 (1 + tanh(c (z + 0.044715 z^3))), c = sqrt(2/pi).
Loss: sum_i w_i (f_i - y_i)^2 / #{w_i > 0}.

The reference has no learned regression (its Laguerre least-squares fit,
src/pricers/lsm.cpp:88-108, is what this network replaces), so this oracle is
checked on its own terms: its backward pass against central finite
differences in FP64 (tests/test_mlp_oracle.py).  With bf16=True it rounds to
BF16 exactly where the GPU feeds the tensor cores (h1, W2, dz2), so the GPU
comparison only has to absorb tanh.approx and FP32 summation order.
"""
from __future__ import annotations

import numpy as np

H = 64
N_PARAMS = 4417
C_GELU = float(np.sqrt(2.0 / np.pi))
W1, B1, W2, B2, W3, B3 = 0, 128, 192, 4288, 4352, 4416


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    f = np.asarray(a, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    u = ((u + 0x7FFF + lsb) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, dtype=np.float64)
    return (p[W1:B1].reshape(H, 2), p[B1:W2], p[W2:B2].reshape(H, H), p[B2:W3], p[W3:B3], p[B3])


def gelu(z):
    t = np.tanh(C_GELU * (z + 0.044715 * z ** 3))
    return 0.5 * z * (1.0 + t), t


def gelu_grad(z, t):
    du = C_GELU * (1.0 + 3.0 * 0.044715 * z * z)
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * du


def forward(p, x0, x1, bf16_tc=False):
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = np.stack([np.asarray(x0, np.float64), np.asarray(x1, np.float64)], axis=1)
    z1 = x @ w1.T + b1
    h1, _ = gelu(z1)
    if bf16_tc:
        h1, w2 = bf16(h1), bf16(w2)
    z2 = h1 @ w2.T + b2
    h2, _ = gelu(z2)
    return h2 @ w3 + b3


def loss_and_grad(p, x0, x1, y, w, bf16_tc=False):
    """Returns (loss, gradient in parameter layout)."""
    w1, b1, w2, b2, w3, b3 = unpack(p)
    x = np.stack([np.asarray(x0, np.float64), np.asarray(x1, np.float64)], axis=1)
    y = np.asarray(y, np.float64)
    wt = np.asarray(w, np.float64)
    n_eff = max(int((wt > 0).sum()), 1)
    z1 = x @ w1.T + b1
    h1, t1 = gelu(z1)
    h1t = bf16(h1) if bf16_tc else h1
    w2t = bf16(w2) if bf16_tc else w2
    z2 = h1t @ w2t.T + b2
    h2, t2 = gelu(z2)
    f = h2 @ w3 + b3
    diff = f - y
    loss = float(np.sum(np.where(wt > 0, diff * diff, 0.0)) / n_eff)
    dy = np.where(wt > 0, 2.0 * diff / n_eff, 0.0)
    g_w3 = dy @ h2
    g_b3 = dy.sum()
    dz2 = dy[:, None] * w3[None, :] * gelu_grad(z2, t2)
    g_b2 = dz2.sum(axis=0)
    dz2t = bf16(dz2) if bf16_tc else dz2
    g_w2 = dz2t.T @ h1t
    dh1 = dz2t @ w2t
    dz1 = dh1 * gelu_grad(z1, t1)
    g_b1 = dz1.sum(axis=0)
    g_w1 = dz1.T @ x
    g = np.zeros(N_PARAMS)
    g[W1:B1] = g_w1.ravel()
    g[B1:W2] = g_b1
    g[W2:B2] = g_w2.ravel()
    g[B2:W3] = g_b2
    g[W3:B3] = g_w3
    g[B3] = g_b3
    return loss, g


def init_params(rng):
    p = np.zeros(N_PARAMS)
    p[W1:B1] = rng.standard_normal(128)
    p[W2:B2] = rng.standard_normal(4096) * np.sqrt(2.0 / 64)
    p[W3:B3] = rng.standard_normal(64) * 0.125
    return p
