"""GPU parity for the GBM path engine, through the C ABI (libmcd_gpu.so).

Bars (stated per test):
  * Philox words: bit-exact against the oracle and the Random123 KATs.
  * FP64 draws: |dz| <= 1e-15 (1+|z|) + 1e-15/phi(z)  (CUDA's erfc/exp vs
    glibc differ in the last ulp; the inverse CDF amplifies that by 1/phi).
  * FP64 prices: within 1e-12 relative of the reference's own values (golden
    vectors) and of the oracle, on identical draws.
  * FP32 prices: within 0.25 standard errors of the FP64 price on the same draws.
  * Bitwise-identical results across launch shapes and between batch and
    single-contract calls.
  * Every product within 3 SE of its analytic price where one exists.
"""
from __future__ import annotations

import ctypes as C
import math

import numpy as np
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

PRICE_REL = 1e-12
SE_REL = 1e-10
FP32_SE_FRACTION = 0.25


def rel_close(a, b, rel):
    return abs(a - b) <= rel * max(abs(a), abs(b), 1e-300)


def test_philox_bit_exact(engine, orc, golden):
    rng = np.random.default_rng(7)
    ctr = rng.integers(0, 2**32, size=(4096, 4), dtype=np.uint64).astype(np.uint32)
    key = rng.integers(0, 2**32, size=(4096, 2), dtype=np.uint64).astype(np.uint32)
    for row in golden["philox"]:  # the reference's KATs first
        ctr = np.vstack([np.array(row["counter"], np.uint32), ctr])
        key = np.vstack([np.array(row["key"], np.uint32), key])
    out = engine.philox(ctr, key)
    for i in range(len(ctr)):
        o = (C.c_uint32 * 4)()
        orc.orc_philox4x32_10((C.c_uint32 * 4)(*ctr[i].tolist()), (C.c_uint32 * 2)(*key[i].tolist()), o)
        assert out[i].tolist() == list(o), i
    for j, row in enumerate(reversed(golden["philox"])):
        assert out[j].tolist() == row["out"]


@pytest.mark.parametrize("seed,path0", [(42, 0), (2**40 + 3, 2**32 - 64), (7, 123456789)])
def test_draws_match_oracle(engine, orc, seed, path0):
    n_paths, n_draws = 128, 40
    z64 = engine.draws(seed, path0, n_paths, 0, n_draws, 0, "fp64")
    z32 = engine.draws(seed, path0, n_paths, 0, n_draws, 0, "fp32")
    u64 = engine.draws(seed, path0, n_paths, 0, n_draws, 1, "fp64")
    worst32 = 0.0
    for p in range(n_paths):
        for d in range(n_draws):
            z = orc.orc_normal_variate(seed, path0 + p, d)
            phi = math.exp(-0.5 * z * z) / math.sqrt(2 * math.pi)
            tol = 1e-15 * (1 + abs(z)) + 1e-15 / phi
            assert abs(z64[p, d] - z) <= tol, (p, d, z64[p, d], z)
            worst32 = max(worst32, abs(z32[p, d] - z) / (1 + abs(z)))
            assert u64[p, d] == orc.orc_uniform_variate(seed, path0 + p, d)
    assert worst32 < 2e-6, worst32


def test_draws_golden(engine, golden):
    for seed, path, d, z, u in golden["draws"]:
        g = engine.draws(seed, path, 1, d, 1, 0, "fp64")[0, 0]
        phi = math.exp(-0.5 * z * z) / math.sqrt(2 * math.pi)
        assert abs(g - z) <= 1e-15 * (1 + abs(z)) + 1e-15 / phi
        assert engine.draws(seed, path, 1, d, 1, 1, "fp64")[0, 0] == u


def _gpu_case(engine, kind, a, precision):
    if kind == "european":
        return engine.monte_carlo_european(*a[:9], antithetic=bool(a[9]), precision=precision)
    if kind == "digital":
        return engine.monte_carlo_digital(*a[:11], antithetic=bool(a[11]), precision=precision)
    if kind == "asian":
        return engine.monte_carlo_asian(*a[:12], antithetic=bool(a[12]),
                                        control_variate=bool(a[13]), precision=precision)
    if kind == "barrier":
        return engine.monte_carlo_barrier(*a[:14], antithetic=bool(a[14]),
                                          brownian_bridge=bool(a[15]), precision=precision)
    return engine.monte_carlo_lookback(*a[:11], antithetic=bool(a[11]), precision=precision)


def test_fp64_matches_reference_golden(engine, golden):
    """Every product / option combination against the reference's own output."""
    for case in golden["mc"]:
        r = _gpu_case(engine, case["kind"], case["args"], "fp64")
        assert r.path_count == case["paths"]
        assert rel_close(r.price, case["price"], PRICE_REL), (case, r)
        assert rel_close(r.standard_error, case["se"], SE_REL), (case, r)


def test_headline_european_fp64(engine, orc):
    r = engine.monte_carlo_european(100, 100, .05, 0, .2, 1, 0, 10**6, 42, precision="fp64")
    assert rel_close(r.price, 10.463094885721839, PRICE_REL)
    assert rel_close(r.standard_error, 0.014739648351400047, SE_REL)
    bsm = orc.orc_bsm(100, 100, .05, 0, .2, 1, 0)
    assert abs(r.price - bsm) < 3 * r.standard_error
    r32 = engine.monte_carlo_european(100, 100, .05, 0, .2, 1, 0, 10**6, 42, precision="fp32")
    assert abs(r32.price - r.price) < FP32_SE_FRACTION * r.standard_error
    assert abs(r32.price - bsm) < 3 * r32.standard_error


def test_fp32_tracks_fp64_on_identical_draws(engine, golden):
    worst = 0.0
    for case in golden["mc"]:
        r64 = _gpu_case(engine, case["kind"], case["args"], "fp64")
        r32 = _gpu_case(engine, case["kind"], case["args"], "fp32")
        se = max(r64.standard_error, 1e-12)
        worst = max(worst, abs(r32.price - r64.price) / se)
        assert abs(r32.price - r64.price) <= FP32_SE_FRACTION * se, (case, r32, r64)
    print(f"max |fp32 - fp64| / SE = {worst:.4f}")


@pytest.mark.parametrize("paths", [0, 1, 2, 4095, 4096, 4097, 3 * 4096 + 17])
def test_ragged_path_counts(engine, orc, paths):
    o = O.options(chunk_count=8)
    ref = orc.orc_mc_barrier(100, 95, 115, .03, .01, .3, 1.5, 1, 0, 1, .25, 7, paths, 99, C.byref(o))
    r = engine.monte_carlo_barrier(100, 95, 115, .03, .01, .3, 1.5, 1, 0, 1, .25, 7, paths, 99)
    assert r.path_count == paths
    if paths == 0:
        assert r.price == 0.0 and r.standard_error == 0.0
        return
    assert rel_close(r.price, ref.price, PRICE_REL)
    if paths >= 2:
        assert rel_close(r.standard_error, ref.standard_error, SE_REL)
    else:
        assert r.standard_error == 0.0


def _mixed_batch(gpu_lib, n=96, seed=3):
    rng = np.random.default_rng(seed)
    c = gpu_lib.contracts(n)
    c["product"] = rng.integers(0, 5, n)
    c["type"] = rng.integers(0, 2, n)
    c["spot"] = 100.0
    c["strike"] = rng.uniform(80, 120, n)
    c["rate"] = rng.uniform(0, .06, n)
    c["vol"] = rng.uniform(.1, .5, n)
    c["time"] = rng.uniform(.25, 2, n)
    c["monitoring_points"] = rng.integers(1, 40, n)
    c["path_count"] = rng.integers(0, 20000, n)
    c["seed"] = 42 + np.arange(n)
    c["direction"] = rng.integers(0, 2, n)
    c["knock"] = rng.integers(0, 2, n)
    c["barrier"] = np.where(c["direction"] == 0, 100 * (1 + rng.uniform(.05, .3, n)),
                            100 * (1 - rng.uniform(.05, .3, n)))
    c["strike_style"] = rng.integers(0, 2, n)
    c["average_style"] = rng.integers(0, 2, n)
    c["digital_style"] = rng.integers(0, 2, n)
    c["antithetic"] = rng.integers(0, 2, n)
    c["brownian_bridge"] = rng.integers(0, 2, n)
    c["control_variate"] = rng.integers(0, 2, n)
    return c


def _orc_contract(orc, row):
    oc = O.Contract()
    for name in row.dtype.names:
        setattr(oc, name, row[name].item())
    out = O.McResult()
    orc.orc_price_batch(C.byref(oc), 1, 1, 8, C.byref(out))
    return out


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batch_equals_single_calls_and_oracle(engine, gpu_lib, orc, precision):
    c = _mixed_batch(gpu_lib)
    batch = engine.price_batch(c, precision)
    singles = np.concatenate([engine.price_batch(c[i:i + 1], precision) for i in range(len(c))])
    assert batch.tobytes() == singles.tobytes()
    for i in range(len(c)):
        ref = _orc_contract(orc, c[i])
        assert batch["path_count"][i] == ref.path_count
        if precision == "fp64":
            assert rel_close(batch["price"][i], ref.price, PRICE_REL), (i, c[i], batch[i], ref.price)
        else:
            assert abs(batch["price"][i] - ref.price) <= FP32_SE_FRACTION * max(ref.standard_error, 1e-12), i


@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_bitwise_identical_across_launch_shapes(engine, gpu_lib, precision):
    c = _mixed_batch(gpu_lib, n=64, seed=11)
    saved = engine.launch_shape(precision)
    outs = []
    try:
        for variant, ctas in [(0, 1), (1, 0), (2, 3), (3, 0), (4, 5), (1, 16), (0, 7)]:
            engine.set_launch_shape(precision, variant, ctas)
            outs.append(engine.price_batch(c, precision).tobytes())
    finally:
        engine.set_launch_shape(precision, saved[0], 0)
    assert all(o == outs[0] for o in outs)


def test_analytic_oracles_within_three_se(engine, orc):
    # European and digital vs closed forms; barrier in+out = vanilla on the same draws.
    r = engine.monte_carlo_european(100, 110, .03, .01, .25, .5, 1, 400000, 5, precision="fp32")
    assert abs(r.price - orc.orc_bsm(100, 110, .03, .01, .25, .5, 1)) < 3 * r.standard_error
    r = engine.monte_carlo_digital(100, 95, .05, 0, .2, 1, 0, 0, 1.0, 400000, 5, precision="fp32")
    assert abs(r.price - orc.orc_digital_analytic(100, 95, .05, 0, .2, 1, 0, 0, 1.0)) < 3 * r.standard_error
    for prec in ("fp64", "fp32"):
        for direction, h in ((0, 120.0), (1, 85.0)):
            ins = engine.monte_carlo_barrier(100, 100, h, .05, 0, .25, 1, 0, direction, 0, 0, 50,
                                             100000, 8, precision=prec)
            outs = engine.monte_carlo_barrier(100, 100, h, .05, 0, .25, 1, 0, direction, 1, 0, 50,
                                              100000, 8, precision=prec)
            never = 1e12 if direction == 0 else 1e-12
            vanilla = engine.monte_carlo_barrier(100, 100, never, .05, 0, .25, 1, 0, direction, 1,
                                                 0, 50, 100000, 8, precision=prec)
            # in + out pays the vanilla on every path (rebate 0)
            assert abs(ins.price + outs.price - vanilla.price) <= 1e-12 * vanilla.price
            assert ins.price > 0 and outs.price > 0
    # Geometric Asian with many dates approaches Kemna-Vorst (continuous monitoring).
    r = engine.monte_carlo_asian(100, 100, .05, 0, .2, 1, 0, 0, 1, 400, 200000, 9, precision="fp32")
    kv = orc.orc_kemna_vorst(100, 100, .05, 0, .2, 1, 0)
    assert abs(r.price - kv) < 3 * r.standard_error + 0.02


def test_invalid_arguments_are_rejected(engine, gpu_lib):
    with pytest.raises(gpu_lib.McdError):
        engine.monte_carlo_european(-1, 100, .05, 0, .2, 1, 0, 1000, 1)
    with pytest.raises(gpu_lib.McdError):
        engine.monte_carlo_asian(100, 100, .05, 0, .2, 1, 0, 0, 0, 0, 1000, 1)
    with pytest.raises(gpu_lib.McdError):
        engine.monte_carlo_european(100, 100, .05, 0, float("nan"), 1, 0, 1000, 1)
    with pytest.raises(gpu_lib.McdError):
        engine.monte_carlo_barrier(100, 100, 0, .05, 0, .2, 1, 0, 0, 0, 0, 5, 100, 1)
    c = gpu_lib.contracts(1)
    c["product"] = 9
    with pytest.raises(gpu_lib.McdError):
        engine.price_batch(c)
    # the context stays usable after a rejected call
    assert engine.monte_carlo_european(100, 100, .05, 0, .2, 1, 0, 1000, 1).path_count == 1000
