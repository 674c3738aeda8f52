"""The ``mcd`` Python module (derivative-pricing_gb300/mcd.py): the reference
module's names, signatures, enums and result shapes (bindings/python/src/
module.cpp:64-293), checked the way the reference's own Python smoke tests
check its module (bindings/python/tests/test_smoke.py): every product prices,
Monte Carlo agrees with the closed forms, result objects expose exactly the
attributes the reference exposes, and pricing releases the GIL.

The closed-form tests run on CPU; everything that prices by simulation is
marked ``gpu``."""
from __future__ import annotations

import math
import threading
import time

import pytest


@pytest.fixture(scope="module")
def mcd(gpu_lib):
    import mcd as module
    return module


# -- CPU: closed forms, enums, argument checks -----------------------------------------

def test_enums_and_constants(mcd):
    assert int(mcd.OptionType.Call) == 0 and int(mcd.OptionType.Put) == 1
    assert int(mcd.BarrierDirection.Down) == 1 and int(mcd.BarrierKnock.Out) == 1
    assert int(mcd.StrikeStyle.Floating) == 1 and int(mcd.AverageStyle.Geometric) == 1
    assert int(mcd.DigitalStyle.AssetOrNothing) == 1
    assert mcd.HAS_NEON is False
    assert mcd.SOBOL_MAX_DIMENSIONS == 256
    o = mcd.McOptions()
    assert (o.antithetic, o.control_variate, o.brownian_bridge, o.num_threads) == (False, False, False, 1)


def test_closed_forms_through_the_module(mcd):
    c = mcd.black_scholes_merton(100, 100, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call)
    assert abs(c - 10.450583572185565) < 1e-12
    assert abs(mcd.forward_price(100, 0.05, 0.02, 1.0) - 100 * math.exp(0.03)) < 1e-12
    tree = mcd.crr_binomial(100, 100, 0.05, 0.0, 0.2, 1.0, 2000, mcd.OptionType.Call)
    assert abs(tree.price - c) < 0.01
    assert tree.up_factor * tree.down_factor == pytest.approx(1.0, abs=1e-15)
    assert 0.0 < tree.risk_neutral_probability < 1.0
    # keyword defaults of the reference bindings: rebate = 0, cash_amount = 1
    ko = mcd.reiner_rubinstein(100, 100, 120, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call,
                               mcd.BarrierDirection.Up, mcd.BarrierKnock.Out)
    ki = mcd.reiner_rubinstein(100, 100, 120, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call,
                               mcd.BarrierDirection.Up, mcd.BarrierKnock.In, rebate=0.0)
    assert abs(ko + ki - c) < 1e-10
    d1 = mcd.digital(100, 100, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call, mcd.DigitalStyle.CashOrNothing)
    d2 = mcd.digital(100, 100, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call, mcd.DigitalStyle.CashOrNothing, 2.0)
    assert d2 == pytest.approx(2.0 * d1, rel=1e-15)


def test_heston_semi_analytic_published_value(mcd):
    # Lewis (2019) reference price for kappa 4, theta 0.25, xi 1, rho -0.5, v0 0.04,
    # r 0.01, q 0.02, T 1, K = S0 = 100 (the case tests/heston_test.cpp:30-51 pins).
    p = mcd.HestonParams()
    p.spot, p.rate, p.carry_yield, p.time = 100.0, 0.01, 0.02, 1.0
    p.v0, p.kappa, p.theta, p.xi, p.rho = 0.04, 4.0, 0.25, 1.0, -0.5
    assert abs(mcd.heston_semi_analytic(p, 100.0, mcd.OptionType.Call) - 16.070154917028834) < 1e-6


def test_qmc_asian_rejects_dimensions_above_the_cap(mcd):
    # checked in the binding before any device work (module.cpp:263-280)
    for bad in (0, mcd.SOBOL_MAX_DIMENSIONS + 1):
        with pytest.raises(ValueError):
            mcd.qmc_sobol_asian(100, 100, 0.05, 0.02, 0.25, 1.0, mcd.OptionType.Call,
                                mcd.StrikeStyle.Fixed, bad, 10_000)


def test_no_broken_estimator_is_offered(mcd):
    assert not hasattr(mcd, "pathwise_digital_delta_naive_and_broken")


# -- GPU: Monte Carlo through the module -----------------------------------------------

@pytest.mark.gpu
def test_every_product_prices(mcd):
    n, seed = 100_000, 42
    C = mcd.OptionType.Call
    results = [
        mcd.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, C, n, seed),
        mcd.monte_carlo_digital(100, 100, 0.05, 0.0, 0.2, 1.0, C, mcd.DigitalStyle.CashOrNothing, 1.0, n, seed),
        mcd.monte_carlo_asian(100, 100, 0.05, 0.0, 0.2, 1.0, C, mcd.StrikeStyle.Fixed,
                              mcd.AverageStyle.Geometric, 12, n, seed),
        mcd.monte_carlo_barrier(100, 100, 120, 0.05, 0.0, 0.2, 1.0, C, mcd.BarrierDirection.Up,
                                mcd.BarrierKnock.Out, 0.0, 20, n, seed),
        mcd.monte_carlo_lookback(100, 100, 0.05, 0.0, 0.2, 1.0, C, mcd.StrikeStyle.Floating, 20, n, seed),
    ]
    for r in results:
        assert r.standard_error > 0.0 and r.path_count == n


@pytest.mark.gpu
def test_european_against_black_scholes_and_options(mcd):
    C = mcd.OptionType.Call
    bs = mcd.black_scholes_merton(100, 100, 0.05, 0.0, 0.2, 1.0, C)
    mc = mcd.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, C, 500_000, 42)
    assert abs(mc.price - bs) < 3.0 * mc.standard_error
    anti = mcd.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, C, 500_000, 42, mcd.McOptions(antithetic=True))
    assert anti.standard_error < mc.standard_error and abs(anti.price - bs) < 3.0 * anti.standard_error
    # the control variate is respected by the arithmetic Asian only
    o = mcd.McOptions()
    o.control_variate = True
    plain = mcd.monte_carlo_asian(100, 100, 0.05, 0.0, 0.2, 1.0, C, mcd.StrikeStyle.Fixed,
                                  mcd.AverageStyle.Arithmetic, 12, 200_000, 7)
    cv = mcd.monte_carlo_asian(100, 100, 0.05, 0.0, 0.2, 1.0, C, mcd.StrikeStyle.Fixed,
                               mcd.AverageStyle.Arithmetic, 12, 200_000, 7, o)
    assert cv.standard_error < 0.2 * plain.standard_error


@pytest.mark.gpu
def test_lsm_and_fd_greeks(mcd):
    r = mcd.monte_carlo_lsm_american(100, 100, 0.05, 0.0, 0.25, 1.0, mcd.OptionType.Put, 20, 50_000, 7)
    assert r.price > 0.0 and r.standard_error >= 0.0
    assert not hasattr(r, "policy")
    bumps = mcd.default_bump_sizes(100, 0.2, 1.0)
    g = mcd.finite_difference_european(100, 100, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call, 300_000, 42, bumps)
    assert 0.0 < g.delta < 1.0 and g.vega > 0.0


@pytest.mark.gpu
def test_likelihood_ratio_result_shapes(mcd):
    C = mcd.OptionType.Call
    lr = mcd.likelihood_ratio_european(100, 100, 0.05, 0.0, 0.2, 1.0, C, 300_000, 42)
    assert 0.0 < lr.delta.value < 1.0 and lr.delta.standard_error > 0.0
    assert lr.theta is not None
    dig = mcd.likelihood_ratio_digital(100, 100, 0.05, 0.0, 0.2, 1.0, C, mcd.DigitalStyle.CashOrNothing,
                                       1.0, 200_000, 7)
    assert dig.gamma.standard_error > 0.0
    bar = mcd.likelihood_ratio_barrier(100, 100, 120, 0.05, 0.0, 0.2, 1.0, C, mcd.BarrierDirection.Up,
                                       mcd.BarrierKnock.Out, 0.0, 50, 100_000, 11)
    assert bar.gamma.standard_error > 0.0 and bar.theta is None


@pytest.mark.gpu
def test_lr_gamma_beats_fd_gamma_at_the_digital_strike(mcd):
    s, k, r, q, v, t = 100.0, 100.0, 0.05, 0.0, 0.25, 1.0
    n, seed = 200_000, 7
    C, cash = mcd.OptionType.Call, mcd.DigitalStyle.CashOrNothing
    lr = mcd.likelihood_ratio_digital(s, k, r, q, v, t, C, cash, 1.0, n, seed)
    h = mcd.default_bump_sizes(s, v, t).spot
    up, mid, dn = (mcd.monte_carlo_digital(x, k, r, q, v, t, C, cash, 1.0, n, seed) for x in (s + h, s, s - h))
    fd_se = math.sqrt(up.standard_error ** 2 + 4 * mid.standard_error ** 2 + dn.standard_error ** 2) / h ** 2
    assert lr.gamma.standard_error < fd_se


@pytest.mark.gpu
def test_pathwise_result_shapes(mcd):
    pw = mcd.pathwise_european(100, 100, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call, 300_000, 42)
    assert 0.0 < pw.delta.value < 1.0 and pw.delta.standard_error > 0.0
    assert not hasattr(pw, "gamma") and not hasattr(pw, "theta")
    pa = mcd.pathwise_asian(100, 100, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call, mcd.StrikeStyle.Fixed,
                            mcd.AverageStyle.Arithmetic, 12, 100_000, 42)
    assert pa.delta.standard_error > 0.0


@pytest.mark.gpu
def test_qmc_through_the_module(mcd):
    C = mcd.OptionType.Call
    bs = mcd.black_scholes_merton(100, 100, 0.05, 0.02, 0.2, 1.0, C)
    e = mcd.qmc_sobol_european(100, 100, 0.05, 0.02, 0.2, 1.0, C, 200_000)
    assert abs(e.price - bs) < 0.02 and not hasattr(e, "standard_error")
    mc = mcd.monte_carlo_asian(100, 100, 0.05, 0.02, 0.25, 1.0, C, mcd.StrikeStyle.Fixed,
                               mcd.AverageStyle.Arithmetic, 7, 100_000, 42)
    a = mcd.qmc_sobol_asian(100, 100, 0.05, 0.02, 0.25, 1.0, C, mcd.StrikeStyle.Fixed, 7, 100_000)
    assert abs(a.price - mc.price) < 3.0 * mc.standard_error + 0.1
    # beyond the reference's 7 dimensions
    wide = mcd.qmc_sobol_asian(100, 100, 0.05, 0.02, 0.25, 1.0, C, mcd.StrikeStyle.Fixed, 250, 100_000)
    assert wide.price > 0.0


@pytest.mark.gpu
def test_heston_qe_through_the_module(mcd):
    p = mcd.HestonParams()
    p.spot, p.rate, p.carry_yield, p.time = 100.0, 0.01, 0.02, 1.0
    p.v0, p.kappa, p.theta, p.xi, p.rho = 0.04, 4.0, 0.25, 1.0, -0.5
    exact = mcd.heston_semi_analytic(p, 100.0, mcd.OptionType.Call)
    mc = mcd.heston_qe_european(p, 100.0, mcd.OptionType.Call, 50, 100_000, 42)
    assert abs(mc.price - exact) < 3.0 * mc.standard_error
    a = mcd.heston_qe_european(p, 100.0, mcd.OptionType.Call, 20, 10_000, 7)
    b = mcd.heston_qe_european(p, 100.0, mcd.OptionType.Call, 20, 10_000, 7)
    assert a.price == b.price


@pytest.mark.gpu
def test_benchmark_harness(mcd):
    out = mcd.benchmark_european(100, 100, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call, 200_000, 42, mcd.McOptions())
    for key in ("price", "standard_error", "path_count", "elapsed_seconds", "paths_per_second", "simd_enabled"):
        assert key in out
    assert out["elapsed_seconds"] > 0.0 and out["paths_per_second"] > 0.0
    assert out["path_count"] == 200_000 and out["simd_enabled"] == mcd.HAS_NEON
    ref = mcd.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, mcd.OptionType.Call, 200_000, 42)
    assert out["price"] == ref.price


@pytest.mark.gpu
def test_precision_is_per_thread(mcd):
    C = mcd.OptionType.Call
    fp64 = mcd.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, C, 1_000_000, 42)
    got = {}

    def worker():
        mcd.set_precision("fp32")
        got["fp32"] = mcd.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, C, 1_000_000, 42)

    th = threading.Thread(target=worker)
    th.start()
    th.join()
    again = mcd.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, C, 1_000_000, 42)
    assert again.price == fp64.price                      # this thread stayed FP64
    assert got["fp32"].price != fp64.price                # the worker priced in FP32
    assert abs(got["fp32"].price - fp64.price) < fp64.standard_error


@pytest.mark.gpu
def test_pricing_releases_the_gil(mcd):
    # A Python thread keeps counting while a long GPU call runs on another: with
    # the GIL held for the call the counter would stall for its whole duration.
    C = mcd.OptionType.Call
    mcd.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, C, 1 << 20, 1)   # context + graph warm-up
    stop = threading.Event()
    ticks = []

    def counter():
        while not stop.is_set():
            ticks.append(time.perf_counter())
            time.sleep(0.0005)

    th = threading.Thread(target=counter)
    th.start()
    time.sleep(0.01)
    t0 = time.perf_counter()
    for seed in range(4):
        mcd.monte_carlo_barrier(100, 100, 130, 0.05, 0.0, 0.2, 1.0, C, mcd.BarrierDirection.Up,
                                mcd.BarrierKnock.Out, 0.0, 252, 1 << 22, seed)
    t1 = time.perf_counter()
    stop.set()
    th.join()
    inside = [x for x in ticks if t0 <= x <= t1]
    gaps = [b - a for a, b in zip(inside, inside[1:])]
    assert t1 - t0 > 0.02, "the calls were too short to test anything"
    assert len(inside) > 10 and max(gaps) < 0.5 * (t1 - t0)
