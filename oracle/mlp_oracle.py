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


# ---------------------------------------------------------------------------
# The fit on node tables (derivative-pricing_gb300/csrc/lsm_mlp_nodes.cu).
# At a date the features are functions of u = ln(S/K) alone; they are tabled
# at nodes u_i = lo + i h and every path uses f(u) = (1 - t) F_i + t F_{i+1}
# (u in bin i at fraction t; u outside the grid uses the end bin, t clamped).
# ---------------------------------------------------------------------------
T_SCALE = 65536.0      # t as an integer of 16 bits
Y_SCALE = 16777216.0   # y / y_bound as an integer of 24 bits


def locate(u, lo, h, n_nodes):
    """Bin and fraction of each u (the kernel's float arithmetic is FP32; here FP64)."""
    x = np.clip((np.asarray(u, dtype=np.float64) - lo) / h, 0.0, n_nodes - 1.0)
    i = np.minimum(x.astype(np.int64), n_nodes - 2)
    t = np.minimum(x - i, 1.0)
    return i, t


def gram_direct(F, i, t, y):
    """Gram matrix of [f | 1 | y] built path by path from interpolated features F[n_nodes, k]."""
    f = (1.0 - t)[:, None] * F[i] + t[:, None] * F[i + 1]
    X = np.c_[f, np.ones(len(t)), y]
    return X.T @ X


def bin_moments(i, t, y, y_bound, n_nodes):
    """The per-bin integer moments the binned pass accumulates: n, sum tq, sum tq^2,
    sum yq, sum tq yq with tq = round(t 2^16), yq = round(y / y_bound 2^24) clamped."""
    tq = np.rint(np.asarray(t) * T_SCALE).astype(np.int64)
    yq = np.clip(np.rint(np.asarray(y) / y_bound * Y_SCALE), -Y_SCALE, Y_SCALE).astype(np.int64)
    m = np.zeros((5, n_nodes - 1), dtype=np.int64)
    np.add.at(m[0], i, 1)
    np.add.at(m[1], i, tq)
    np.add.at(m[2], i, tq * tq)
    np.add.at(m[3], i, yq)
    np.add.at(m[4], i, tq * yq)
    return m


def gram_from_moments(F, m, y_bound):
    """lsm_mlp_gram_slices' formula: G = sum over bins of Saa F_i F_i^T + Sab (F_i F_{i+1}^T
    + F_{i+1} F_i^T) + Sbb F_{i+1} F_{i+1}^T, the right-hand side sum Say F_i + Sby F_{i+1},
    with Saa = sum (1-t)^2, Sab = sum t(1-t), Sbb = sum t^2, Say = sum (1-t) y, Sby = sum t y;
    the constant feature is a column of ones in F (the y^2 entry is not formed)."""
    n = m[0].astype(np.float64)
    st = m[1] / T_SCALE
    stt = m[2] / T_SCALE ** 2
    sy = m[3] * (y_bound / Y_SCALE)
    sty = m[4] * (y_bound / (T_SCALE * Y_SCALE))
    saa, sab, sbb, say, sby = n - 2 * st + stt, st - stt, stt, sy - sty, sty
    Fc = np.c_[F, np.ones(len(F))]
    A, B = Fc[:-1], Fc[1:]
    k = Fc.shape[1]
    G = np.zeros((k + 1, k + 1))
    G[:k, :k] = (A.T * saa) @ A + (A.T * sab) @ B + (B.T * sab) @ A + (B.T * sbb) @ B
    G[:k, k] = A.T @ say + B.T @ sby
    G[k, :k] = G[:k, k]
    return G
