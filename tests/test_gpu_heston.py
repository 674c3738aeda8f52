"""GPU parity for Heston QE (src/pricers/heston.cpp:91-156) through the C ABI.

Bars: FP64 within 1e-12 relative of the reference's own outputs (golden) and of
the oracle on identical draws; FP32 within 0.25 SE of FP64 on the same draws;
the multi-strike batch equals one reference call per (set, strike); prices
within 3 SE of the semi-analytic price (Lewis's published parameters).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

LEWIS = [100.0, .01, .02, .04, 4.0, .25, 1.0, -.5, 1.0]


def test_fp64_matches_reference_golden(engine, golden):
    for case in golden["heston"]:
        r = engine.heston_qe_european(case["params"], case["strike"], case["type"], case["steps"],
                                      case["paths"], case["seed"], precision="fp64")
        assert r.path_count == case["paths"]
        assert abs(r.price - case["price"]) <= 1e-12 * abs(case["price"]), (case, r)
        assert abs(r.standard_error - case["se"]) <= 1e-10 * case["se"]


def test_batch_equals_per_strike_oracle_calls(engine, orc):
    rng = np.random.default_rng(3)
    sets = []
    for _ in range(3):
        sets.append([100.0, .03, 0.0, rng.uniform(.01, .09), rng.uniform(.5, 3), rng.uniform(.02, .09),
                     rng.uniform(.2, 1.0), rng.uniform(-.9, -.3), 1.0])
    strikes = np.linspace(70, 130, 7)
    paths, steps, seed = 3000, 24, 77
    got = engine.heston_qe_batch(sets, strikes, 0, steps, paths, seed, "fp64")
    got32 = engine.heston_qe_batch(sets, strikes, 0, steps, paths, seed, "fp32")
    for i, s in enumerate(sets):
        hp = O.HestonParams(*s)
        for j, k in enumerate(strikes):
            ref = orc.orc_heston_qe_european(C.byref(hp), k, 0, steps, paths, seed)
            assert got["path_count"][i, j] == paths
            assert abs(got["price"][i, j] - ref.price) <= 1e-12 * max(abs(ref.price), 1e-300), (i, j)
            assert abs(got32["price"][i, j] - ref.price) <= 0.25 * ref.standard_error, (i, j)


@pytest.mark.parametrize("n_strikes", [1, 64, 200])
def test_strike_counts_and_ragged_paths(engine, orc, n_strikes):
    strikes = np.linspace(60, 140, n_strikes)
    paths = 4096 + 37
    got = engine.heston_qe_batch([LEWIS], strikes, 1, 10, paths, 5, "fp64")
    hp = O.HestonParams(*LEWIS)
    for j in sorted({0, n_strikes // 2, n_strikes - 1}):
        ref = orc.orc_heston_qe_european(C.byref(hp), strikes[j], 1, 10, paths, 5)
        assert abs(got["price"][0, j] - ref.price) <= 1e-12 * abs(ref.price)
        assert abs(got["standard_error"][0, j] - ref.standard_error) <= 1e-10 * ref.standard_error


def test_within_three_se_of_semi_analytic(engine, orc):
    hp = O.HestonParams(*LEWIS)
    strikes = np.array([80.0, 100.0, 120.0])
    got = engine.heston_qe_batch([LEWIS], strikes, 0, 100, 1 << 18, 11, "fp32")
    for j, k in enumerate(strikes):
        sa = orc.orc_heston_semi_analytic(C.byref(hp), k, 0)
        assert abs(got["price"][0, j] - sa) < 3 * got["standard_error"][0, j] + 0.01, (k, got[0, j], sa)


def test_invalid_heston_arguments(engine, gpu_lib):
    bad = list(LEWIS)
    bad[6] = 0.0  # xi = 0 divides K0..K2
    with pytest.raises(gpu_lib.McdError):
        engine.heston_qe_european(bad, 100, 0, 10, 100, 1)
    with pytest.raises(gpu_lib.McdError):
        engine.heston_qe_batch([LEWIS], np.linspace(50, 150, 300), 0, 10, 100, 1)
