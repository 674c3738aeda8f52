"""Frozen-boundary American Greeks (mcd_lsm_frozen_greeks, mcd_lsm_greeks_batch).

The reference's recipe (tests/lsm_test.cpp:138-185): fit the policy once, then
reprice against the frozen policy (src/pricers/lsm.cpp:151-213) at bumped
inputs with the same seed.  The GPU streams all scenarios of a path in one pass
with no stored paths; these tests pin that pass to the replay, bit for bit, and
the replay to the oracle:
  * base scenario == the fitted LSM price (same paths, same decisions);
  * each bumped scenario == mcd_lsm_reprice_frozen at the bumped inputs;
  * FP64 scenarios within 1e-12 of the oracle's replay (oracle/mcd_oracle.c);
  * the batch form == fitting and replaying each contract alone;
  * delta and vega within a few standard errors of the CRR tree's.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PUT = 1


def fit(engine, args, precision):
    return engine.monte_carlo_lsm_american(*args, precision=precision, policy=True)


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_scenarios_are_the_frozen_replays(engine, precision):
    s, k, r, q, v, t, n, paths, seed = 36.0, 40.0, 0.06, 0.0, 0.2, 1.0, 50, 100_000, 42
    args = (s, k, r, q, v, t, PUT, n, paths, seed)
    res, co, has = fit(engine, args, precision)
    assert not res.exercise_at_inception
    hs, hv = 0.4, 0.002
    g = engine.lsm_frozen_greeks(*args, co, has, False, spot_bump=hs, vol_bump=hv, precision=precision)
    assert g["price"][0] == res.price
    assert g["path_count"] == paths
    bumped = [(s + hs, v), (s - hs, v), (s, v + hv), (s, v - hv)]
    for (sb, vb), scen in zip(bumped, g["scenario"]):
        rep = engine.reprice_against_frozen_policy(sb, k, r, q, vb, t, PUT, n, paths, seed, co, has, False,
                                                   precision=precision)
        assert scen == rep, (sb, vb, scen, rep)
    up, dn, vu, vd = g["scenario"]
    assert g["delta"][0] == (up - dn) / (2 * hs)
    assert g["gamma"][0] == (up - 2.0 * res.price + dn) / (hs * hs)
    assert g["vega"][0] == (vu - vd) / (2 * hv)
    assert g["delta"][1] > 0 and g["gamma"][1] > 0 and g["vega"][1] > 0


def test_fp64_scenarios_match_oracle(engine, orc):
    s, k, r, q, v, t, n, paths, seed = 100.0, 100.0, 0.05, 0.01, 0.25, 1.0, 20, 20_000, 7
    args = (s, k, r, q, v, t, PUT, n, paths, seed)
    res, co, has = fit(engine, args, "fp64")
    hs, hv = 0.5, 0.005
    g = engine.lsm_frozen_greeks(*args, co, has, False, spot_bump=hs, vol_bump=hv, precision="fp64")
    co = np.ascontiguousarray(co, dtype=np.float64)
    has = np.ascontiguousarray(has, dtype=np.uint8)
    for (sb, vb), got in zip([(s, v), (s + hs, v), (s - hs, v), (s, v + hv), (s, v - hv)],
                             [g["price"][0], *g["scenario"]]):
        want = orc.orc_lsm_reprice_frozen(sb, k, r, q, vb, t, PUT, n, paths, seed,
                                          co.ctypes.data_as(C.POINTER(C.c_double)),
                                          has.ctypes.data_as(C.POINTER(C.c_uint8)), 0)
        assert abs(got - want) <= 1e-12 * abs(want), (sb, vb, got, want)


def test_batch_equals_single_contract_calls(engine, gpu_lib):
    rng = np.random.default_rng(5)
    c = np.zeros(6, dtype=gpu_lib.LSM_CONTRACT_DTYPE)
    c["spot"] = rng.uniform(34, 46, 6)
    c["strike"] = 40.0
    c["rate"] = 0.06
    c["vol"] = rng.uniform(0.15, 0.4, 6)
    c["time"] = rng.uniform(0.5, 2.0, 6)
    c["type"] = PUT
    c["monitoring_points"] = rng.integers(10, 60, 6)
    c["path_count"] = rng.integers(20_000, 80_000, 6)
    c["seed"] = np.arange(6) + 100
    for precision in ("fp64", "fp32"):
        batch = engine.lsm_greeks_batch(c, 0.01, 0.02, precision=precision)
        for i, row in enumerate(c):
            args = (float(row["spot"]), 40.0, 0.06, 0.0, float(row["vol"]), float(row["time"]), PUT,
                    int(row["monitoring_points"]), int(row["path_count"]), int(row["seed"]))
            res, co, has = fit(engine, args, precision)
            one = engine.lsm_frozen_greeks(*args, co, has, res.exercise_at_inception,
                                           spot_bump=0.01 * args[0], vol_bump=0.02 * args[4],
                                           precision=precision)
            for name in ("price", "delta", "gamma", "vega", "scenario"):
                assert np.array_equal(batch[i][name], one[name]), (precision, i, name)


@pytest.mark.parametrize("spot", [36.0, 40.0, 44.0])
def test_delta_and_vega_against_crr_tree(engine, gpu_lib, spot):
    k, r, q, v, t, n, paths, seed = 40.0, 0.06, 0.0, 0.2, 1.0, 50, 1 << 18, 11
    args = (spot, k, r, q, v, t, PUT, n, paths, seed)
    res, co, has = fit(engine, args, "fp64")
    hs, hv = 0.01 * spot, 0.01 * v
    g = engine.lsm_frozen_greeks(*args, co, has, res.exercise_at_inception, spot_bump=hs, vol_bump=hv)

    def tree(sp, vol):
        return gpu_lib.crr_binomial_american(sp, k, r, q, vol, t, 2000, PUT)

    delta = (tree(spot + hs, v) - tree(spot - hs, v)) / (2 * hs)
    vega = (tree(spot, v + hv) - tree(spot, v - hv)) / (2 * hv)
    # a 50-date Bermudan against continuous exercise: a small bias on top of the noise
    assert abs(g["delta"][0] - delta) < 5 * g["delta"][1] + 0.01, (g["delta"], delta)
    assert abs(g["vega"][0] - vega) < 5 * g["vega"][1] + 0.03 * abs(vega), (g["vega"], vega)


def test_exercise_at_inception_freezes_to_intrinsic(engine):
    s, k, r, q, v, t, n, paths, seed = 20.0, 40.0, 0.06, 0.0, 0.2, 1.0, 20, 10_000, 3
    args = (s, k, r, q, v, t, PUT, n, paths, seed)
    res, co, has = fit(engine, args, "fp64")
    assert res.exercise_at_inception
    g = engine.lsm_frozen_greeks(*args, co, has, True, spot_bump=0.5, vol_bump=0.01)
    assert g["price"][0] == 20.0 and g["price"][1] == 0.0
    assert g["delta"][0] == -1.0 and g["gamma"][0] == 0.0 and g["vega"][0] == 0.0
    assert g["exercise_at_inception"] == 1


def test_invalid_bumps(engine, gpu_lib):
    args = (36.0, 40.0, 0.06, 0.0, 0.2, 1.0, PUT, 10, 1000, 1)
    res, co, has = fit(engine, args, "fp64")
    for hs, hv in ((0.0, 0.01), (36.0, 0.01), (0.1, 0.0), (0.1, 0.2)):
        with pytest.raises(gpu_lib.McdError):
            engine.lsm_frozen_greeks(*args, co, has, False, spot_bump=hs, vol_bump=hv)
    c = np.zeros(1, dtype=gpu_lib.LSM_CONTRACT_DTYPE)
    c["spot"], c["strike"], c["vol"], c["time"], c["monitoring_points"], c["path_count"] = 36, 40, .2, 1, 10, 1000
    with pytest.raises(gpu_lib.McdError):
        engine.lsm_greeks_batch(c, 1.0, 0.01)
