"""Closed forms, CRR lattices and the semi-analytic Heston price of libmcd_gpu.so
(host FP64, no GPU) against the values the reference itself computed
(tests/golden/reference_vectors.json, "analytic"; generated by
tests/golden/make_golden.py from src/pricers/analytic.cpp, binomial.cpp and
heston.cpp).  The functions keep the reference's operation order, so the bar is
a few ulps, not a modelling tolerance."""
from __future__ import annotations

import math

import pytest

REL = 1e-13          # same formula, same operation order: rounding of erfc/exp/log only
REL_HESTON = 1e-10   # complex logarithms and 256 characteristic-function calls


def close(a, b, rel):
    return math.isclose(a, b, rel_tol=rel, abs_tol=rel)


@pytest.fixture(scope="module")
def analytic(golden):
    return golden["analytic"]


def test_black_scholes_merton(gpu_lib, analytic):
    for *args, t, want in analytic["bsm"]:
        assert close(gpu_lib.black_scholes_merton(*args, t), want, REL)


def test_black76(gpu_lib, analytic):
    for *args, t, want in analytic["black76"]:
        assert close(gpu_lib.black76(*args, t), want, REL)


def test_kemna_vorst(gpu_lib, analytic):
    for *args, t, want in analytic["kemna_vorst"]:
        assert close(gpu_lib.kemna_vorst(*args, t), want, REL)


def test_reiner_rubinstein_all_sixteen_branches(gpu_lib, analytic):
    rows = analytic["reiner_rubinstein"]
    branches = {(r[7], r[8], r[9], r[1] > r[2]) for r in rows}
    assert len(branches) == 16  # call/put x up/down x in/out x strike above/below barrier
    for s, k, h, r, q, v, t, typ, d, kn, rebate, want in rows:
        got = gpu_lib.reiner_rubinstein(s, k, h, r, q, v, t, typ, d, kn, rebate)
        assert close(got, want, REL), (typ, d, kn, k > h, got, want)


def test_lookbacks(gpu_lib, analytic):
    for *args, t, want in analytic["lookback_fixed"]:
        assert close(gpu_lib.lookback_fixed_strike(*args, t), want, REL)
    for *args, t, want in analytic["lookback_floating"]:
        assert close(gpu_lib.lookback_floating_strike(*args, t), want, REL)


def test_digital(gpu_lib, analytic):
    for s, k, r, q, v, t, typ, style, cash, want in analytic["digital"]:
        assert close(gpu_lib.digital(s, k, r, q, v, t, typ, style, cash), want, REL)
    # default cash amount 1 (module.cpp:188-191)
    s, k, r, q, v, t, typ, style, cash, want = analytic["digital"][0]
    if style == gpu_lib.CASH_OR_NOTHING:
        assert close(gpu_lib.digital(s, k, r, q, v, t, typ, style), want / cash, REL)


def test_forwards_and_futures(gpu_lib, analytic):
    for *args, want in analytic["forward_price"]:
        assert close(gpu_lib.forward_price(*args), want, REL)
    for *args, want in analytic["forward_value"]:
        assert close(gpu_lib.forward_value(*args), want, REL)
    for a, b, want in analytic["futures_mtm"]:
        assert gpu_lib.futures_mark_to_market(a, b) == want


def test_crr_lattices(gpu_lib, analytic):
    for s, k, r, q, v, t, n, typ, price, p, u, d in analytic["crr_european"]:
        res = gpu_lib.crr_binomial(s, k, r, q, v, t, n, typ)
        assert close(res.price, price, 1e-12)
        assert close(res.risk_neutral_probability, p, REL)
        assert close(res.up_factor, u, REL) and close(res.down_factor, d, REL)
    for *args, n, typ, want in analytic["crr_american"]:
        assert close(gpu_lib.crr_binomial_american(*args, n, typ), want, 1e-12)
    with pytest.raises(gpu_lib.McdError):
        gpu_lib.crr_binomial(100, 100, 0.05, 0, 0.2, 1, 0, gpu_lib.CALL)
    assert math.isnan(gpu_lib.crr_binomial_american(100, 100, 0.05, 0, 0.2, 1, 0, gpu_lib.PUT))


def test_heston_semi_analytic(gpu_lib, analytic):
    for p9, strike, typ, want in analytic["heston_semi_analytic"]:
        params = gpu_lib.HestonParams(*p9)
        assert close(gpu_lib.heston_semi_analytic(params, strike, typ), want, REL_HESTON)


def test_put_call_parity_of_closed_forms(gpu_lib):
    s, k, r, q, v, t = 100.0, 97.0, 0.04, 0.015, 0.27, 1.3
    c = gpu_lib.black_scholes_merton(s, k, r, q, v, t, gpu_lib.CALL)
    p = gpu_lib.black_scholes_merton(s, k, r, q, v, t, gpu_lib.PUT)
    assert abs((c - p) - (s * math.exp(-q * t) - k * math.exp(-r * t))) < 1e-12
    # in + out = vanilla for a zero rebate (Reiner-Rubinstein, every direction)
    for d in (gpu_lib.UP, gpu_lib.DOWN):
        h = 120.0 if d == gpu_lib.UP else 80.0
        ki = gpu_lib.reiner_rubinstein(s, k, h, r, q, v, t, gpu_lib.CALL, d, gpu_lib.IN)
        ko = gpu_lib.reiner_rubinstein(s, k, h, r, q, v, t, gpu_lib.CALL, d, gpu_lib.OUT)
        assert abs(ki + ko - c) < 1e-10


def test_bermudan_lattice_brackets():
    """mcd_crr_binomial_bermudan (no reference counterpart): with an exercise
    date on every tree step it is the reference's American CRR price; with one
    date (t = 0 only) it is max(intrinsic, European); otherwise in between."""
    import mcd_gpu as M
    args = (36.0, 40.0, 0.06, 0.0, 0.2, 1.0)
    amer = M.crr_binomial_american(*args, 2000, 1)
    assert abs(M.crr_binomial_bermudan(*args, 2000, 1, 1) - amer) <= 1e-12 * amer
    euro = M.crr_binomial(*args, 2000, 1).price
    assert abs(M.crr_binomial_bermudan(*args, 1, 2000, 1) - max(4.0, euro)) <= 1e-12
    berm = M.crr_binomial_bermudan(*args, 50, 40, 1)
    assert euro < berm < amer
    import math
    assert math.isnan(M.crr_binomial_bermudan(*args, 0, 10, 1))
