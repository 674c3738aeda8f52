"""GPU checks of the Sobol quasi-Monte Carlo engine (derivative-pricing_gb300/csrc/qmc.cu).

Bars:
  * Device Sobol coordinates equal the reference's (golden vectors, dims 0..6)
    and the oracle's extension (dims 7..255) exactly.
  * FP64 QMC European and arithmetic Asian prices equal the reference's
    (golden, src/pricers/qmc.cpp) to 1e-12 relative; only the order of the
    final sum differs.  Beyond the reference's 7 dimensions the oracle
    restatement (same bridge, same Sobol extension) is the bar.
  * FP32 agrees with FP64 to 1e-4 relative; QMC prices of every batch product
    agree with FP64 Monte Carlo within 4 of its standard errors; a contract
    priced alone equals its batch result bit for bit.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

import mcd_gpu as G

pytestmark = pytest.mark.gpu


def test_sobol_points_match_reference_and_oracle(engine, golden, orc):
    table = golden["sobol"]
    for d in range(7):
        ref = np.array(table[str(d)])
        got = engine.sobol_points(d, 1, 0, len(ref))[:, 0]
        assert (got == ref).all(), d
    idx = [1, 2, 3, 5, 8, 13, 1000, 65535, 65536, 123457, (1 << 31) + 7]
    for d in (7, 8, 31, 100, 200, 255):
        for i in idx:
            got = engine.sobol_points(d, 1, i, 1)[0, 0]
            assert got == orc.orc_sobol_point(d, i), (d, i)
    block = engine.sobol_points(0, 256, 1, 64)
    assert block.shape == (64, 256) and (block > 0).all() and (block < 1).all()


def test_qmc_matches_reference(engine, golden):
    for row in golden["qmc_european"]:
        *args, paths, price = row
        got = engine.qmc_sobol_european(*args, paths, precision="fp64")
        assert abs(got - price) <= 1e-12 * abs(price), (got, price)
    for row in golden["qmc_asian"]:
        s, k, r, q, v, t, ty, style, n, paths, price = row
        got = engine.qmc_sobol_asian(s, k, r, q, v, t, ty, style, n, paths, precision="fp64")
        assert abs(got - price) <= 1e-12 * abs(price) + 1e-13, (n, style, got, price)


@pytest.mark.parametrize("n", [8, 13, 50, 252])
def test_qmc_asian_beyond_seven_dims_matches_oracle(engine, orc, n):
    for ty, style in ((0, 0), (1, 1)):
        got = engine.qmc_sobol_asian(100.0, 95.0, 0.04, 0.01, 0.3, 1.5, ty, style, n, 5000, precision="fp64")
        ref = orc.orc_qmc_sobol_asian(100.0, 95.0, 0.04, 0.01, 0.3, 1.5, ty, style, n, 5000)
        assert abs(got - ref) <= 1e-12 * abs(ref) + 1e-13, (n, got, ref)
        f32 = engine.qmc_sobol_asian(100.0, 95.0, 0.04, 0.01, 0.3, 1.5, ty, style, n, 5000, precision="fp32")
        assert abs(f32 - ref) <= 1e-4 * abs(ref) + 1e-6, (n, f32, ref)


def _mix():
    rows = []

    def add(product, type_=0, **kw):
        c = dict(product=product, type=type_, spot=100.0, strike=100.0, rate=0.03, carry_yield=0.0, vol=0.3,
                 time=1.0, cash_amount=1.0, path_count=1 << 16, seed=11, monitoring_points=1)
        c.update(kw)
        rows.append(c)

    add(G.EUROPEAN, 0)
    add(G.DIGITAL, 1)
    add(G.ASIAN, 0, monitoring_points=64, strike_style=0, average_style=0)
    add(G.ASIAN, 1, monitoring_points=100, strike_style=1, average_style=1)
    add(G.BARRIER, 0, monitoring_points=52, barrier=130.0, direction=0, knock=1)
    add(G.BARRIER, 1, monitoring_points=30, barrier=80.0, direction=1, knock=0)
    add(G.LOOKBACK, 0, monitoring_points=40, strike_style=0)
    add(G.LOOKBACK, 1, monitoring_points=252, strike_style=1)
    arr = np.zeros(len(rows), dtype=G.CONTRACT_DTYPE)
    for i, r in enumerate(rows):
        for k, v in r.items():
            arr[i][k] = v
    return arr


def test_qmc_batch_against_monte_carlo(engine):
    arr = _mix()
    q64 = engine.qmc_batch(arr, precision="fp64")
    q32 = engine.qmc_batch(arr, precision="fp32")
    mc = arr.copy()
    mc["path_count"] = 1 << 20
    ref = engine.price_batch(mc, precision="fp64")
    for i in range(len(arr)):
        assert q64["standard_error"][i] == 0.0
        assert q64["path_count"][i] == arr["path_count"][i]
        assert abs(q64["price"][i] - ref["price"][i]) < 4 * ref["standard_error"][i] + 2e-3, (i, q64[i], ref[i])
        assert abs(q32["price"][i] - q64["price"][i]) <= 2e-4 * abs(q64["price"][i]) + 1e-5, (i, q32[i], q64[i])


def test_qmc_european_converges_to_black_scholes(engine, orc):
    bsm = orc.orc_bsm(100.0, 100.0, 0.05, 0.0, 0.2, 1.0, 0)
    got = engine.qmc_sobol_european(100.0, 100.0, 0.05, 0.0, 0.2, 1.0, 0, 1 << 22, precision="fp32")
    assert abs(got - bsm) < 2e-3, (got, bsm)


def test_qmc_batch_equals_single_and_rejects_unsupported(engine):
    arr = _mix()
    full = engine.qmc_batch(arr, precision="fp32")
    for i in range(len(arr)):
        one = engine.qmc_batch(arr[i:i + 1], precision="fp32")
        assert one.tobytes() == full[i:i + 1].tobytes(), i
    bad = arr[2:3].copy()
    bad["monitoring_points"] = 257
    with pytest.raises(G.McdError):
        engine.qmc_batch(bad)
    bad = arr[2:3].copy()
    bad["control_variate"] = 1
    with pytest.raises(G.McdError):
        engine.qmc_batch(bad)
