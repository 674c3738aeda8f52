"""GPU parity for Longstaff-Schwartz (src/pricers/lsm.cpp:62-213) through the C ABI.

Bars:
  * FP64: price within 1e-12 relative of the reference's own output (golden),
    standard error within 1e-10 -- the GPU solves the same least-squares problem
    by Cholesky-QR2 instead of a sequential Householder QR; the coefficients are
    determined by the data only up to the problem's conditioning (the
    reference's own Householder moves them by ~1e-9 relative when the rows are
    reordered, tests/test_lsm_conditioning.py), the fitted continuation values
    agree to 1e-8 of the coefficient scale, and every exercise decision
    coincides.  The full-size grid is tests/test_gpu_lsm_grid.py.
  * Frozen-policy repricing with the reference's own policy: within 1e-12.
  * FP32 paths: within 0.5 SE of the FP64 price on the same draws.
  * Within 3 SE of the 4000-step CRR American tree (tests/lsm_test.cpp:78-98:
    its grid, path count and seed), FP64 and FP32, and American call without
    dividends == Black-Scholes (lsm_test.cpp:26-38).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


def test_fp64_matches_reference_golden(engine, golden):
    for case in golden["lsm"]:
        s, k, r, q, v, t, ty, n, paths, seed = case["args"]
        res, co, has = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, seed,
                                                       precision="fp64", policy=True)
        assert res.path_count == paths
        assert abs(res.price - case["price"]) <= 1e-12 * case["price"], (case["args"], res.price)
        assert abs(res.standard_error - case["se"]) <= 1e-10 * case["se"]
        assert res.exercise_at_inception == case["inception"]
        assert has.tolist() == case["has"]
        ref = np.array(case["coefficients"]).reshape(-1, 4)
        for d in range(1, n):
            if not has[d]:
                continue
            scale = np.abs(ref[d]).sum()
            assert np.abs(co[d] - ref[d]).max() <= 1e-7 * scale, (d, co[d], ref[d])
            # fitted continuation values on a grid of x = S/K
            for x in np.linspace(0.5, 1.0, 6):
                e = np.exp(-x / 2)
                b = np.array([e, e * (1 - x), e * (1 - 2 * x + .5 * x * x),
                              e * (1 - 3 * x + 1.5 * x * x - x ** 3 / 6)])
                assert abs(b @ co[d] - b @ ref[d]) <= 1e-8 * scale


def test_frozen_policy_reprice_matches_oracle(engine, orc, golden):
    case = golden["lsm"][0]
    s, k, r, q, v, t, ty, n, paths, seed = case["args"]
    co = np.array(case["coefficients"])
    has = np.array(case["has"], dtype=np.uint8)
    for bump in (0.0, 0.5, -0.5):
        gpu = engine.reprice_against_frozen_policy(s + bump, k, r, q, v, t, ty, n, paths, seed, co,
                                                   has, False, precision="fp64")
        ref = orc.orc_lsm_reprice_frozen(s + bump, k, r, q, v, t, ty, n, paths, seed,
                                         co.ctypes.data_as(C.POINTER(C.c_double)),
                                         has.ctypes.data_as(C.POINTER(C.c_uint8)), 0)
        assert abs(gpu - ref) <= 1e-12 * ref
    # replayed inception exercise returns the intrinsic value
    assert engine.reprice_against_frozen_policy(30, 40, r, q, v, t, 1, n, 1000, seed, co, has, True) == 10.0


def test_fp32_tracks_fp64(engine):
    for (s, k, v, t) in [(36, 40, .2, 1), (44, 40, .4, 2), (40, 40, .2, 1)]:
        r64 = engine.monte_carlo_lsm_american(s, k, .06, 0, v, t, 1, 50, 1 << 16, 42, precision="fp64")
        r32 = engine.monte_carlo_lsm_american(s, k, .06, 0, v, t, 1, 50, 1 << 16, 42, precision="fp32")
        assert abs(r32.price - r64.price) <= 0.5 * r64.standard_error, (s, k, v, t, r32, r64)


def test_against_binomial_tree(engine, orc):
    """tests/lsm_test.cpp:78-98 as the reference runs it: 50 dates, 100,000
    paths, seed 909, a 4000-step CRR tree, strictly within 3 SE -- on the FP64
    path (the reference's arithmetic) and on the FP32 batch."""
    grid = [(100, 100, .05, 0, .25, 1.0, 1), (100, 80, .05, 0, .25, 1.0, 1),
            (100, 120, .05, 0, .25, 1.0, 1), (100, 100, .05, .03, .30, .5, 1),
            (100, 100, .05, .03, .30, .5, 0), (100, 100, .03, .06, .20, 2.0, 1)]
    c = np.zeros(len(grid), dtype=__import__("mcd_gpu").LSM_CONTRACT_DTYPE)
    for i, (s, k, r, q, v, t, ty) in enumerate(grid):
        c[i] = (s, k, r, q, v, t, ty, 50, 100000, 909)
    out32 = engine.lsm_batch(c, "fp32")
    for i, (s, k, r, q, v, t, ty) in enumerate(grid):
        tree = orc.orc_crr_binomial_american(s, k, r, q, v, t, 4000, ty)
        r64 = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, 50, 100000, 909, precision="fp64")
        assert abs(r64.price - tree) < 3 * r64.standard_error, (grid[i], r64, tree)
        assert abs(out32["price"][i] - tree) < 3 * out32["standard_error"][i], (grid[i], out32[i], tree)
    call = engine.monte_carlo_lsm_american(100, 100, .05, 0, .25, 1, 0, 50, 100000, 909, precision="fp32")
    assert abs(call.price - orc.orc_bsm(100, 100, .05, 0, .25, 1, 0)) < 3 * call.standard_error


def test_batch_with_uneven_dates_equals_single_calls(engine, gpu_lib):
    rng = np.random.default_rng(4)
    n = 7
    c = np.zeros(n, dtype=gpu_lib.LSM_CONTRACT_DTYPE)
    c["spot"] = rng.uniform(36, 44, n)
    c["strike"] = 40
    c["rate"] = .06
    c["vol"] = rng.uniform(.2, .4, n)
    c["time"] = rng.uniform(.5, 2, n)
    c["type"] = 1
    c["monitoring_points"] = [1, 2, 10, 37, 50, 3, 100]
    c["path_count"] = [1023, 1025, 5000, 8192, 3000, 777, 2048]
    c["seed"] = 42 + np.arange(n)
    for prec in ("fp64", "fp32"):
        batch = engine.lsm_batch(c, prec)
        for i in range(n):
            one = engine.lsm_batch(c[i:i + 1], prec)
            assert one.tobytes() == batch[i:i + 1].tobytes(), (prec, i)


def test_edge_cases_match_oracle(engine, orc):
    # one date (no regression), ragged paths, deep out-of-the-money (too few ITM paths)
    for (s, k, ty, n, paths) in [(40, 40, 1, 1, 1000), (36, 40, 1, 5, 1025), (80, 40, 1, 10, 2000),
                                 (40, 40, 0, 4, 3)]:
        res = engine.monte_carlo_lsm_american(s, k, .06, 0, .2, 1, ty, n, paths, 7, precision="fp64")
        ref = orc.orc_lsm_american(s, k, .06, 0, .2, 1, ty, n, paths, 7, None, None, None)
        assert abs(res.price - ref.price) <= 1e-12 * max(ref.price, 1e-300) + 1e-15, (s, k, n, paths, res, ref.price)


def test_invalid_lsm_arguments(engine, gpu_lib):
    with pytest.raises(gpu_lib.McdError):
        engine.monte_carlo_lsm_american(36, 40, .06, 0, .2, 1, 1, 0, 1000, 1)
    with pytest.raises(gpu_lib.McdError):
        engine.monte_carlo_lsm_american(36, -40, .06, 0, .2, 1, 1, 10, 1000, 1)


def test_frozen_boundary_delta_has_lower_variance_than_naive_refit(engine):
    # tests/lsm_test.cpp:138-185 on the GPU: delta by CRN spot bumps of the
    # frozen base policy against delta by re-fitting LSM at each bumped spot,
    # over 40 seeds; the frozen estimator must have the smaller spread.
    s, k, r, q, v, t, h = 100.0, 100.0, 0.05, 0.0, 0.25, 1.0, 0.1
    paths, n = 5000, 20
    frozen, naive = [], []
    for trial in range(40):
        seed = 42 + trial * 1013
        base, co, hq = engine.monte_carlo_lsm_american(s, k, r, q, v, t, 1, n, paths, seed, policy=True)
        up = engine.reprice_against_frozen_policy(s + h, k, r, q, v, t, 1, n, paths, seed, co, hq,
                                                  base.exercise_at_inception)
        dn = engine.reprice_against_frozen_policy(s - h, k, r, q, v, t, 1, n, paths, seed, co, hq,
                                                  base.exercise_at_inception)
        frozen.append((up - dn) / (2 * h))
        nu = engine.monte_carlo_lsm_american(s + h, k, r, q, v, t, 1, n, paths, seed).price
        nd = engine.monte_carlo_lsm_american(s - h, k, r, q, v, t, 1, n, paths, seed).price
        naive.append((nu - nd) / (2 * h))
    sf, sn = float(np.std(frozen, ddof=1)), float(np.std(naive, ddof=1))
    print(f"frozen-boundary delta sd {sf:.5f}, naive refit sd {sn:.5f}, ratio {sn / sf:.2f}")
    assert sf < sn
    assert -0.6 < float(np.mean(frozen)) < -0.2  # an at-the-money American put's delta


def test_fp32_ill_conditioned_first_pass(engine, orc):
    """A put whose raw Laguerre Gram matrix is not numerically positive
    definite on some date of the FP32 path: the first-pass Cholesky is
    retried with a small diagonal shift (shifted Cholesky QR) instead of
    dropping the preconditioner, so the FP32 price stays with the FP64 price
    and the tree (without the retry it fell 27 standard errors short)."""
    args = (39.57831059016732, 40.0, 0.06, 0.0, 0.2668022683651664, 1.1610222409416884, 1, 93, 1 << 18, 1468)
    r32 = engine.monte_carlo_lsm_american(*args, precision="fp32")
    r64 = engine.monte_carlo_lsm_american(*args, precision="fp64")
    tree = orc.orc_crr_binomial_american(*args[:6], 2000, 1)
    assert abs(r32.price - r64.price) < 0.25 * r64.standard_error, (r32.price, r64.price)
    assert abs(r64.price - tree) < 3 * r64.standard_error + 0.02, (r64.price, tree)
