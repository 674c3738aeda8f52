"""Longstaff-Schwartz at full size against the reference's own prices.

The American-put grid (S0 in {36..44}, K=40, r=.06, sigma in {.2,.4}, T in
{1,2}, 50 dates, 2^20 paths, seed 42+i) priced by the reference's
monte_carlo_lsm_american (src/pricers/lsm.cpp:62-149) compiled from source
(tests/golden/make_lsm_grid_golden.py -> lsm_grid_2p20.json).  The first put is
S0=36, sigma=.2, T=1, seed 42: 4.476383949663612.

Bars:
  * FP64 batch (mcd_lsm_batch): every price within 1e-12 relative of the
    reference, standard errors within 1e-10, the same inception decisions and
    the same dates with a regression.  A single exercise decision that differed
    on one of the 2^20 paths would move a price by ~1e-6 relative, so this also
    shows that every decision on every date coincides.
  * The fitted continuation values (what the decisions compare against)
    agree with the reference's over the in-the-money range to 1e-10 of the
    coefficient scale; the coefficients themselves are determined by the data
    only up to the least-squares conditioning (tests/test_lsm_conditioning.py).
  * FP32 paths with the QR regression: within 0.1 SE of the reference.
"""
from __future__ import annotations

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def grid(gpu_lib):
    with open(os.path.join(HERE, "golden", "lsm_grid_2p20.json")) as f:
        g = json.load(f)
    c = np.array([tuple(p["args"]) for p in g["puts"]], dtype=gpu_lib.LSM_CONTRACT_DTYPE)
    return c, g["puts"]


def _laguerre(x):
    e = np.exp(-x / 2)
    return np.stack([e, e * (1 - x), e * (1 - 2 * x + .5 * x * x), e * (1 - 3 * x + 1.5 * x * x - x ** 3 / 6)], -1)


def test_fp64_grid_matches_reference_to_1e12(engine, grid):
    c, puts = grid
    assert c["path_count"][0] == 1 << 20 and c["monitoring_points"][0] == 50
    assert puts[0]["price"] == 4.476383949663612
    out = engine.lsm_batch(c, "fp64", "qr")
    rel = np.abs(out["price"] - [p["price"] for p in puts]) / [p["price"] for p in puts]
    print("FP64 grid, max relative difference from the reference:", rel.max())
    for i, p in enumerate(puts):
        assert out["path_count"][i] == 1 << 20
        assert abs(out["price"][i] - p["price"]) <= 1e-12 * p["price"], (i, out["price"][i], p["price"])
        assert abs(out["standard_error"][i] - p["se"]) <= 1e-10 * p["se"], (i, out["standard_error"][i], p["se"])
        assert bool(out["exercise_at_inception"][i]) == bool(p["inception"])


def test_fp64_policies_match_reference(engine, grid):
    c, puts = grid
    worst_fit = 0.0
    for p in puts:
        s, k, r, q, v, t, ty, n, paths, seed = p["args"]
        res, co, has = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, seed,
                                                       precision="fp64", policy=True)
        assert abs(res.price - p["price"]) <= 1e-12 * p["price"]
        assert has.tolist() == p["has"]
        ref = np.array(p["coefficients"]).reshape(-1, 4)
        for d in range(1, n):
            if not has[d]:
                continue
            # S/K over the put's in-the-money side where date d has paths
            # (5 standard deviations of the log-spot below its mean)
            td = d * t / n
            lo = s * np.exp((r - q - v * v / 2) * td - 5 * v * np.sqrt(td)) / k
            b = _laguerre(np.linspace(max(lo, 0.3), 1.0, 26))
            scale = np.abs(ref[d]).sum()
            fit = np.abs(b @ (co[d] - ref[d])).max() / scale
            worst_fit = max(worst_fit, fit)
            assert fit <= 1e-10, (p["args"], d, fit)
    print("largest continuation-value difference / coefficient scale:", worst_fit)


def test_fp32_qr_grid_tracks_reference(engine, grid):
    c, puts = grid
    out = engine.lsm_batch(c, "fp32", "qr")
    err = np.abs(out["price"] - [p["price"] for p in puts]) / [p["se"] for p in puts]
    print("FP32 QR grid, error in reference standard errors: max", err.max(), "mean", err.mean())
    assert err.max() <= 0.1
