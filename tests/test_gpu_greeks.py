"""GPU checks of the sensitivity engine (derivative-pricing_gb300/csrc/greeks.cu).

Bars:
  * FP64 likelihood-ratio and pathwise Greeks equal the reference's own values
    (golden vectors from src/greeks/*.cpp) to 1e-10 relative; the reference
    accumulates sequentially, the GPU in slabs, so only the summation order
    differs.
  * FP64 finite-difference European Greeks (nine CRN re-prices in one batch)
    equal the reference's to 1e-8 relative.
  * Batched FP64 finite differences equal central differences of the oracle's
    common-random-number re-prices (same seed, bumped contract) for every
    product the engine covers; the price output equals mcd_price_batch's bit
    for bit in both precisions.
  * FP32 (one log-path, differential vol states) agrees with FP64 within a
    fraction of the Monte Carlo standard error, and every estimator of a
    European call lands within 4 SE of Black-Scholes.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import mcd_gpu as G
import oracle as O

pytestmark = pytest.mark.gpu

REL = 1e-10


def close(a, b, rel=REL, abs_=1e-13):
    return abs(a - b) <= abs_ + rel * abs(b)


def test_lr_matches_reference(engine, golden):
    lr = golden["lr"]
    a = lr["european"]["args"]
    r = engine.likelihood_ratio_european(*a, precision="fp64")
    got = [r.delta.value, r.delta.standard_error, r.gamma.value, r.gamma.standard_error, r.vega.value,
           r.vega.standard_error, r.rho.value, r.rho.standard_error, r.theta.value, r.theta.standard_error]
    for x, y in zip(got, lr["european"]["out"]):
        assert close(x, y), (got, lr["european"]["out"])
    assert r.has_theta == 1
    a = lr["digital"]["args"]  # (..., type, digital style, cash, paths, seed)
    r = engine.likelihood_ratio_digital(*a, precision="fp64")
    got = [r.delta.value, r.delta.standard_error, r.gamma.value, r.gamma.standard_error, r.vega.value,
           r.vega.standard_error, r.rho.value, r.rho.standard_error, r.theta.value, r.theta.standard_error]
    for x, y in zip(got, lr["digital"]["out"]):
        assert close(x, y), (got, lr["digital"]["out"])
    a = lr["barrier"]["args"]
    r = engine.likelihood_ratio_barrier(*a, precision="fp64")
    got = [r.delta.value, r.delta.standard_error, r.gamma.value, r.gamma.standard_error, r.vega.value,
           r.vega.standard_error, r.rho.value, r.rho.standard_error]
    for x, y in zip(got, lr["barrier"]["out"]):
        assert close(x, y), (got, lr["barrier"]["out"])
    assert r.has_theta == 0


def test_pathwise_matches_reference(engine, golden):
    pw = golden["pathwise"]
    r = engine.pathwise_european(*pw["european"]["args"], precision="fp64")
    got = [r.delta.value, r.delta.standard_error, r.vega.value, r.vega.standard_error, r.rho.value,
           r.rho.standard_error]
    for x, y in zip(got, pw["european"]["out"]):
        assert close(x, y), (got, pw["european"]["out"])
    for key in ("asian_00", "asian_01", "asian_10", "asian_11"):
        r = engine.pathwise_asian(*pw[key]["args"], precision="fp64")
        got = [r.delta.value, r.delta.standard_error, r.vega.value, r.vega.standard_error, r.rho.value,
               r.rho.standard_error]
        for x, y in zip(got, pw[key]["out"]):
            assert close(x, y), (key, got, pw[key]["out"])


def test_fd_european_matches_reference(engine, golden):
    fd = golden["fd_european"]
    b = G.BumpSizes(*fd["bumps"])
    r = engine.finite_difference_european(*fd["args"], bumps=b, precision="fp64")
    got = [r.delta, r.gamma, r.vega, r.theta, r.rho]
    for x, y in zip(got, fd["greeks"]):
        assert close(x, y, rel=1e-8), (got, fd["greeks"])
    d = engine.default_bump_sizes(100.0, 0.2, 1.0)
    assert (d.spot, d.vol, d.rate, d.time) == (1.0, 0.002, 0.01, 0.01)


def _contracts():
    rows = []

    def add(product, type_=0, **kw):
        c = dict(product=product, type=type_, spot=100.0, strike=100.0, rate=0.05, carry_yield=0.01,
                 vol=0.25, time=1.0, cash_amount=1.0, path_count=12000, seed=7 + len(rows),
                 monitoring_points=1)
        c.update(kw)
        rows.append(c)

    add(G.EUROPEAN, 0)
    add(G.EUROPEAN, 1, strike=95.0)
    add(G.DIGITAL, 0, digital_style=0)
    add(G.DIGITAL, 1, digital_style=1)
    add(G.ASIAN, 0, monitoring_points=24, strike_style=0, average_style=0)
    add(G.ASIAN, 1, monitoring_points=17, strike_style=1, average_style=0)
    add(G.ASIAN, 0, monitoring_points=24, strike_style=0, average_style=1)
    add(G.ASIAN, 1, monitoring_points=9, strike_style=1, average_style=1)
    add(G.BARRIER, 0, monitoring_points=32, barrier=125.0, direction=0, knock=1)
    add(G.BARRIER, 1, monitoring_points=20, barrier=85.0, direction=1, knock=0, rebate=1.5)
    add(G.LOOKBACK, 0, monitoring_points=16, strike_style=0)
    add(G.LOOKBACK, 1, monitoring_points=16, strike_style=1)
    arr = np.zeros(len(rows), dtype=G.CONTRACT_DTYPE)
    for i, r in enumerate(rows):
        for k, v in r.items():
            arr[i][k] = v
    return arr


def _oracle_prices(orc, arr):
    out = (O.McResult * len(arr))()
    cs = (O.Contract * len(arr)).from_buffer_copy(arr.tobytes())
    orc.orc_price_batch(cs, len(arr), 1, 8, out)
    return np.array([o.price for o in out])


@pytest.mark.parametrize("rel_bump", [1e-2, 1e-4])
def test_batched_fd_matches_oracle_reprices(engine, orc, rel_bump):
    arr = _contracts()
    res = engine.greeks_batch(arr, rel_bump, rel_bump, precision="fp64")
    bumped = []
    for field, sgn in (("spot", 1), ("spot", -1), ("vol", 1), ("vol", -1)):
        b = arr.copy()
        b[field] = arr[field] + sgn * (rel_bump * arr[field])  # the kernel's S0 +/- h
        bumped.append(_oracle_prices(orc, b))
    base = _oracle_prices(orc, arr)
    hs, hv = rel_bump * arr["spot"], rel_bump * arr["vol"]
    delta = (bumped[0] - bumped[1]) / (2 * hs)
    gamma = (bumped[0] - 2 * base + bumped[1]) / (hs * hs)
    vega = (bumped[2] - bumped[3]) / (2 * hv)
    for i in range(len(arr)):
        assert close(res["price"][i][0], base[i], rel=1e-12), (i, res["price"][i][0], base[i])
        # the oracle's differences of means against the GPU's means of differences
        assert close(res["fd_delta"][i][0], delta[i], rel=1e-8, abs_=1e-9), (i, res["fd_delta"][i], delta[i])
        assert close(res["fd_vega"][i][0], vega[i], rel=1e-8, abs_=1e-8), (i, res["fd_vega"][i], vega[i])
        tol_g = 1e-12 * max(abs(base[i]), 1.0) / float(hs[i]) ** 2 * 8
        assert abs(res["fd_gamma"][i][0] - gamma[i]) <= tol_g + 1e-8 * abs(gamma[i]), (i, res["fd_gamma"][i], gamma[i])
    assert (res["path_count"] == arr["path_count"]).all()


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_price_output_is_the_pricer_bitwise(engine, precision):
    arr = _contracts()
    res = engine.greeks_batch(arr, 1e-4, 1e-4, precision=precision)
    ref = engine.price_batch(arr, precision=precision)
    assert (res["price"][:, 0] == ref["price"]).all()
    assert (res["price"][:, 1] == ref["standard_error"]).all()


def test_fp32_agrees_with_fp64(engine):
    arr = _contracts()
    arr["path_count"] = 40000
    r64 = engine.greeks_batch(arr, 1e-4, 1e-4, precision="fp64")
    r32 = engine.greeks_batch(arr, 1e-4, 1e-4, precision="fp32")
    # Discontinuous payoffs (digital, barrier): a path within FP32 rounding of
    # the strike or barrier can land on the other side, and with 1e-4 bumps one
    # such path moves a finite difference by a visible share of its SE.
    jumpy = np.isin(arr["product"], [G.DIGITAL, G.BARRIER])
    for name in ("price", "fd_delta", "fd_vega", "pathwise_delta", "pathwise_vega", "pathwise_rho", "lr_delta",
                 "lr_gamma", "lr_vega", "lr_rho"):
        for i in range(len(arr)):
            if not (r64["defined"][i] >> G.GREEK_NAMES.index(name)) & 1:
                continue
            a, se = r32[name][i]
            b, se64 = r64[name][i]
            f = 1.0 if jumpy[i] else 0.1
            assert abs(a - b) <= f * max(se, se64) + 1e-9 * abs(b) + 1e-12, (name, i, a, b, se)
    # gamma: FD with 1e-4 bumps only sees paths at the kink; same bar where it is smooth
    for i in range(len(arr)):
        a, se = r32["fd_gamma"][i]
        b, _ = r64["fd_gamma"][i]
        f = 1.0 if jumpy[i] else 0.5
        assert abs(a - b) <= f * se + 1e-6 * abs(b) + 1e-9, ("fd_gamma", i, a, b, se)


def test_european_call_estimators_against_black_scholes(engine, orc):
    s, k, r, q, v, t = 100.0, 100.0, 0.05, 0.01, 0.25, 1.0
    arr = np.zeros(1, dtype=G.CONTRACT_DTYPE)
    arr[0]["product"], arr[0]["spot"], arr[0]["strike"], arr[0]["rate"] = G.EUROPEAN, s, k, r
    arr[0]["carry_yield"], arr[0]["vol"], arr[0]["time"] = q, v, t
    arr[0]["path_count"], arr[0]["seed"], arr[0]["monitoring_points"] = 1 << 21, 3, 1
    res = engine.greeks_batch(arr, 1e-2, 1e-2, precision="fp32")[0]
    d1 = (math.log(s / k) + (r - q + 0.5 * v * v) * t) / (v * math.sqrt(t))
    pdf = math.exp(-0.5 * d1 * d1) / math.sqrt(2 * math.pi)
    delta = math.exp(-q * t) * orc.orc_normal_cdf(d1)
    gamma = math.exp(-q * t) * pdf / (s * v * math.sqrt(t))
    vega = s * math.exp(-q * t) * pdf * math.sqrt(t)
    assert abs(res["price"][0] - orc.orc_bsm(s, k, r, q, v, t, 0)) < 4 * res["price"][1]
    for name, exact in (("fd_delta", delta), ("pathwise_delta", delta), ("lr_delta", delta),
                        ("fd_vega", vega), ("pathwise_vega", vega), ("lr_vega", vega),
                        ("fd_gamma", gamma), ("lr_gamma", gamma)):
        val, se = res[name]
        # FD with a 1 % bump carries an O(h^2) bias on top of the noise
        bias = 2e-3 * abs(exact) if name.startswith("fd") else 0.0
        assert abs(val - exact) < 4 * se + bias, (name, val, se, exact)


def test_batch_equals_single_and_rejects_unsupported(engine):
    arr = _contracts()
    full = engine.greeks_batch(arr, 1e-4, 1e-4, precision="fp32")
    for i in (0, 5, 9):
        one = engine.greeks_batch(arr[i:i + 1], 1e-4, 1e-4, precision="fp32")
        assert one.tobytes() == full[i:i + 1].tobytes()
    bad = arr[:1].copy()
    bad["antithetic"] = 1
    with pytest.raises(G.McdError):
        engine.greeks_batch(bad, 1e-4, 1e-4)
    with pytest.raises(G.McdError):
        engine.greeks_batch(arr[:1], 0.0, 1e-4)
