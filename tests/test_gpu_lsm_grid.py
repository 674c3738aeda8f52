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


def test_learned_grid_against_the_exact_bermudan_value(engine, grid, gpu_lib):
    """The learned regression (BF16 tensor-core network, FP32 paths) on the
    full grid, checked against the exact value of the 50-date Bermudan put (CRR
    lattice with exercise at the LSM dates) and against the FP64 QR price.

    * Every learned price within 3 SE of the exact value (as every Monte Carlo
      price here must be of its analytic or lattice oracle), and on average
      no farther from it than the QR regression's.
    * The learned price sits above the FP64 QR price by up to ~1.2 SE.  That
      gap is the better exercise policy, not an error: replayed on fresh paths
      (no foresight), the learned policy earns more than the QR policy on
      every put."""
    c, puts = grid
    M = gpu_lib
    ml = engine.lsm_batch(c, "fp32", "mlp")
    qr = engine.lsm_batch(c, "fp64", "qr")
    se = qr["standard_error"]
    berm = np.array([M.crr_binomial_bermudan(r["spot"], r["strike"], r["rate"], r["carry_yield"], r["vol"], r["time"],
                                             int(r["monitoring_points"]), 100, 1) for r in c])
    z_ml, z_qr = (ml["price"] - berm) / se, (qr["price"] - berm) / se
    gap = (ml["price"] - qr["price"]) / se
    print(f"vs exact Bermudan: learned max|z| {np.abs(z_ml).max():.2f} mean|z| {np.abs(z_ml).mean():.2f}; "
          f"QR max|z| {np.abs(z_qr).max():.2f} mean|z| {np.abs(z_qr).mean():.2f}; "
          f"learned - QR: mean {gap.mean():+.2f} max {gap.max():+.2f} SE")
    assert (ml["reserved"] == 0).all()  # no fallback to QR
    assert np.abs(z_ml).max() < 3.0
    assert np.abs(z_ml).mean() <= np.abs(z_qr).mean() + 0.1
    gains = []
    for i, r in enumerate(c):
        w, has = engine.mlp_policy(i, int(r["monitoring_points"]))
        args = (r["spot"], r["strike"], r["rate"], r["carry_yield"], r["vol"], r["time"], int(r["type"]),
                int(r["monitoring_points"]))
        _, co, hq = engine.monte_carlo_lsm_american(*args, int(r["path_count"]), int(r["seed"]),
                                                    precision="fp64", policy=True)
        fresh = int(r["seed"]) + 10_000_000
        q_oos = engine.reprice_against_frozen_policy(*args, int(r["path_count"]), fresh, co, hq, False, "fp64")
        m_oos = engine.reprice_mlp(*args, int(r["path_count"]), fresh, w, has, "fp32")
        gains.append((m_oos.price - q_oos) / m_oos.standard_error)
    gains = np.array(gains)
    print(f"out of sample, learned - QR policy: min {gains.min():+.2f} mean {gains.mean():+.2f} SE")
    assert (gains > 0).all()
    assert (gap > -0.5).all() and gap.max() < 2.0


def test_learned_per_date_fine_tuning_changes_little(engine, grid):
    """The hidden layers are trained once, on the latest date; every date
    refits the output layer exactly on all its in-the-money paths.  Fine-tuning
    the hidden layers at every date as well (Adam steps warm-started from the
    later date) moves no price by more than a fraction of its SE: the features
    learned once already span each date's continuation value."""
    c, _ = grid
    base = engine.lsm_batch(c, "fp32", "mlp")
    try:
        engine.set_mlp_config(100, 5, 3e-3, 3e-4)
        tuned = engine.lsm_batch(c, "fp32", "mlp")
    finally:
        engine.set_mlp_config()
    d = np.abs(tuned["price"] - base["price"]) / base["standard_error"]
    print(f"per-date fine-tuning (5 steps): max change {d.max():.3f} SE, mean {d.mean():.3f} SE")
    assert d.max() < 0.5 and d.mean() < 0.2


def test_learned_fp32_within_one_se_of_learned_fp64(engine, grid):
    """The learned regression's own FP64 oracle: the same method on FP64 paths
    (FP64 path store, exercise tests and cash flows; the same network and
    fit).  On every put of the full grid the FP32 price is within 1 SE of it
    (measured: at most ~0.06 SE), at 1/35 of its time."""
    c, _ = grid
    f32 = engine.lsm_batch(c, "fp32", "mlp")
    f64 = engine.lsm_batch(c, "fp64", "mlp")
    assert (f32["reserved"] == 0).all() and (f64["reserved"] == 0).all()
    d = np.abs(f32["price"] - f64["price"]) / f64["standard_error"]
    print(f"learned FP32 vs learned FP64: max {d.max():.3f} SE, mean {d.mean():.3f} SE")
    assert d.max() <= 1.0
