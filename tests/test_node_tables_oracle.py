"""The node-table fit of the learned regression restated on the CPU
(oracle/mlp_oracle.py): the Gram matrix the GPU builds from per-bin integer
moments equals the Gram matrix of the interpolated features built path by
path, up to the moments' quantisation (t to 2^-16 of a bin, y to 2^-24 of its
bound), for data shaped like a date of an American put."""
from __future__ import annotations

import numpy as np

import mlp_oracle as M


def test_gram_from_bin_moments_matches_paths():
    rng = np.random.default_rng(3)
    n_nodes, k, paths = 512, 64, 200_000
    F = np.tanh(rng.standard_normal((1, k)) * np.linspace(-3, 0, n_nodes)[:, None] + rng.standard_normal(k))
    lo, hi = -1.4, 0.0
    h = (hi - lo) / (n_nodes - 1)
    u = np.minimum(rng.normal(-0.3, 0.25, paths), -1e-9)   # in-the-money side of a put
    u[:5] = [lo - 0.5, lo, hi, -1e-12, lo + 7.5 * h]       # beyond the grid, its ends, a node
    y = rng.normal(0.02, 0.05, paths)
    i, t = M.locate(u, lo, h, n_nodes)
    G = M.gram_direct(F, i, t, y)
    Gm = M.gram_from_moments(F, M.bin_moments(i, t, y, 1.0, n_nodes), 1.0)
    k1 = k + 1
    scale = np.sqrt(np.outer(np.diag(G[:k1, :k1]), np.diag(G[:k1, :k1])))
    assert np.abs(Gm[:k1, :k1] - G[:k1, :k1]).max() / scale.max() < 1e-5
    rhs_scale = np.sqrt(np.diag(G[:k1, :k1]) * G[k1, k1])
    assert np.max(np.abs(Gm[:k1, k1] - G[:k1, k1]) / rhs_scale) < 1e-5
    assert Gm[k, k] == paths                               # the count is exact


def test_locate_clamps_to_the_end_bins():
    i, t = M.locate(np.array([-10.0, 0.0, 10.0, 0.5]), 0.0, 0.25, 5)
    assert list(i) == [0, 0, 3, 2] and list(t) == [0.0, 0.0, 1.0, 0.0]
