"""Pins the CPU oracle against the reference's own known answers and against
vectors recorded from the reference built from source (CPU only).

Mirrors the reference's tests: Philox KATs (tests/rng_test.cpp:17-39), inverse
CDF vs a Newton root finder (:60-102), Lewis Heston prices at 1e-9
(tests/heston_test.cpp:45-62), and every pricer on fixed seeds.
"""
from __future__ import annotations

import ctypes as C
import math

import pytest

import oracle as O

REL = 1e-13  # libm may differ in the last ulp across machines; bitwise where it does not


def close(a, b, rel=REL, abs_=0.0):
    return abs(a - b) <= max(rel * max(abs(a), abs(b)), abs_)


def test_philox_known_answers(orc, golden):
    for row in golden["philox"]:
        out = (C.c_uint32 * 4)()
        orc.orc_philox4x32_10((C.c_uint32 * 4)(*row["counter"]), (C.c_uint32 * 2)(*row["key"]), out)
        assert list(out) == row["out"]


def test_random123_pi_vector(orc):
    # tests/rng_test.cpp:33-39 (Random123 kat_vectors, "pi digits" case)
    out = (C.c_uint32 * 4)()
    orc.orc_philox4x32_10((C.c_uint32 * 4)(0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344),
                          (C.c_uint32 * 2)(0xA4093822, 0x299F31D0), out)
    assert list(out) == [0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_draws_match_reference(orc, golden):
    for seed, path, d, z, u in golden["draws"]:
        assert close(orc.orc_normal_variate(seed, path, d), z)
        assert orc.orc_uniform_variate(seed, path, d) == u  # pure integer->double, exact


def test_inverse_cdf_vs_newton(orc):
    def newton(u):
        z = 0.0
        for _ in range(100):
            step = (orc.orc_normal_cdf(z) - u) / orc.orc_normal_pdf(z)
            z -= step
            if abs(step) < 1e-15:
                break
        return z

    us, p = [], 1e-9
    while p < 0.5:
        us += [p, 1 - p]
        p *= 3.16227766017
    us.append(0.5)
    assert max(abs(orc.orc_inv_normal_cdf(u) - newton(u)) for u in us) < 1e-9


def test_inverse_cdf_golden(orc, golden):
    for u, z in golden["inv_normal_cdf"]:
        assert close(orc.orc_inv_normal_cdf(u), z)


def _mc(orc, kind, a, chunks):
    if kind == "european":
        o = O.options(antithetic=bool(a[9]), chunk_count=chunks)
        return orc.orc_mc_european(*a[:9], C.byref(o))
    if kind == "digital":
        o = O.options(antithetic=bool(a[11]), chunk_count=chunks)
        return orc.orc_mc_digital(*a[:11], C.byref(o))
    if kind == "asian":
        o = O.options(antithetic=bool(a[12]), control_variate=bool(a[13]), chunk_count=chunks)
        return orc.orc_mc_asian(*a[:12], C.byref(o))
    if kind == "barrier":
        o = O.options(antithetic=bool(a[14]), brownian_bridge=bool(a[15]), chunk_count=chunks)
        return orc.orc_mc_barrier(*a[:14], C.byref(o))
    o = O.options(antithetic=bool(a[11]), chunk_count=chunks)
    return orc.orc_mc_lookback(*a[:11], C.byref(o))


def test_mc_products_match_reference(orc, golden):
    chunks = golden["chunk_count"]
    assert len(golden["mc"]) >= 30
    for case in golden["mc"]:
        r = _mc(orc, case["kind"], case["args"], chunks)
        assert close(r.price, case["price"]), case
        assert close(r.standard_error, case["se"]), case
        assert r.path_count == case["paths"]


def test_headline_european_value(orc):
    # S0=K=100, r=.05, q=0, sigma=.2, T=1, 1e6 paths, seed 42 at 8 chunks.
    o = O.options(chunk_count=8)
    r = orc.orc_mc_european(100, 100, .05, 0, .2, 1, 0, 10**6, 42, C.byref(o))
    assert close(r.price, 10.463094885721839)
    assert abs(r.price - orc.orc_bsm(100, 100, .05, 0, .2, 1, 0)) < 3 * r.standard_error


def test_thread_count_invariance(orc):
    # tests/parallelism_test.cpp: bitwise-identical results across thread counts.
    base = None
    for t in (1, 2, 3, 8):
        o = O.options(num_threads=t, chunk_count=8)
        r = orc.orc_mc_asian(100, 100, .05, 0, .3, 1, 0, 0, 0, 12, 50003, 5, C.byref(o))
        key = (r.price, r.standard_error)
        base = base or key
        assert key == base


def test_lsm_matches_reference(orc, golden):
    for case in golden["lsm"]:
        s, k, r_, q, v, t, ty, n, paths, seed = case["args"]
        co = O.dbuf((n + 1) * 4)
        ho = (C.c_uint8 * (n + 1))()
        inc = C.c_int(0)
        res = orc.orc_lsm_american(s, k, r_, q, v, t, ty, n, paths, seed, co, ho, C.byref(inc))
        assert close(res.price, case["price"], 1e-12)
        assert close(res.standard_error, case["se"], 1e-10)
        assert list(ho) == case["has"]
        for a, b in zip(co, case["coefficients"]):
            assert close(a, b, 1e-9, 1e-12)


def test_heston_matches_reference_and_lewis(orc, golden):
    lewis = {80: 26.774758743998854221, 90: 20.933349000596710388, 100: 16.070154917028834278,
             110: 12.132211516709844868, 120: 9.024913483457835637}
    hp = O.HestonParams(100, .01, .02, .04, 4, .25, 1, -.5, 1)
    for k, v in lewis.items():
        assert abs(orc.orc_heston_semi_analytic(C.byref(hp), k, 0) - v) < 1e-9
    for case in golden["heston"]:
        hp = O.HestonParams(*case["params"])
        r = orc.orc_heston_qe_european(C.byref(hp), case["strike"], case["type"], case["steps"],
                                       case["paths"], case["seed"])
        assert close(r.price, case["price"], 1e-12)
        assert close(orc.orc_heston_semi_analytic(C.byref(hp), case["strike"], case["type"]),
                     case["semi_analytic"], 1e-12)


def test_sobol_and_qmc_match_reference(orc, golden):
    for d, pts in golden["sobol"].items():
        for i, x in enumerate(pts):
            assert orc.orc_sobol_point(int(d), i) == x
    for row in golden["qmc_european"]:
        assert close(orc.orc_qmc_sobol_european(*row[:8]), row[8], 1e-12)
    for row in golden["qmc_asian"]:
        assert close(orc.orc_qmc_sobol_asian(*row[:10]), row[10], 1e-12)


def test_sobol_extension_is_primitive_and_stratified(orc):
    # Dimensions beyond the reference's 7 use further primitive polynomials
    # (LFSR period check as in tests/sobol_test.cpp:19-54) and keep 1-D
    # stratification (:59-82).
    seen = set()
    for d in range(1, O.__dict__.get("SOBOL_DIMS", 256)):
        deg, mask = C.c_uint(), C.c_uint32()
        assert orc.orc_sobol_polynomial(d, C.byref(deg), C.byref(mask)) == 0
        key = (deg.value, mask.value)
        assert key not in seen
        seen.add(key)
        s = deg.value
        poly = (1 << s) | 1
        for j in range(1, s):
            if (mask.value >> (j - 1)) & 1:
                poly |= 1 << (s - j)
        r, period = 1, 0
        while True:
            r <<= 1
            if r & (1 << s):
                r ^= poly
            period += 1
            if r == 1:
                break
        assert period == (1 << s) - 1, (d, s, mask.value)
    for d in (7, 50, 251):
        for k in (1, 2, 4, 6):
            n = 1 << k
            bins = sorted(int(orc.orc_sobol_point(d, i) * n) for i in range(n))
            assert bins == list(range(n))


def test_greeks_match_reference(orc, golden):
    fd = golden["fd_european"]
    b = O.Bumps(*fd["bumps"])
    g = orc.orc_fd_european(*fd["args"], b, golden["chunk_count"])
    for a, e in zip((g.delta, g.gamma, g.vega, g.theta, g.rho), fd["greeks"]):
        assert close(a, e, 1e-10)
    lr = golden["lr"]
    g = orc.orc_lr_european(*lr["european"]["args"])
    vals = [g.delta.value, g.delta.standard_error, g.gamma.value, g.gamma.standard_error,
            g.vega.value, g.vega.standard_error, g.rho.value, g.rho.standard_error,
            g.theta.value, g.theta.standard_error]
    for a, e in zip(vals, lr["european"]["out"]):
        assert close(a, e, 1e-12)
    g = orc.orc_lr_digital(*lr["digital"]["args"])
    assert close(g.gamma.value, lr["digital"]["out"][2], 1e-12)
    g = orc.orc_lr_barrier(*lr["barrier"]["args"])
    assert g.has_theta == 0
    for a, e in zip([g.delta.value, g.delta.standard_error, g.gamma.value, g.gamma.standard_error,
                     g.vega.value, g.vega.standard_error, g.rho.value, g.rho.standard_error],
                    lr["barrier"]["out"]):
        assert close(a, e, 1e-12)
    pw = golden["pathwise"]
    g = orc.orc_pathwise_european(*pw["european"]["args"])
    for a, e in zip([g.delta.value, g.delta.standard_error, g.vega.value, g.vega.standard_error,
                     g.rho.value, g.rho.standard_error], pw["european"]["out"]):
        assert close(a, e, 1e-12)
    for key in ("asian_00", "asian_01", "asian_10", "asian_11"):
        g = orc.orc_pathwise_asian(*pw[key]["args"])
        assert close(g.delta.value, pw[key]["out"][0], 1e-12)
        assert close(g.vega.value, pw[key]["out"][2], 1e-12)


def test_analytic_oracles(orc, golden):
    an = golden["analytic"]
    for row in an["bsm"]:
        assert close(orc.orc_bsm(*row[:7]), row[7], 1e-14)
    for row in an["kemna_vorst"]:
        assert close(orc.orc_kemna_vorst(*row[:7]), row[7], 1e-14)
    for row in an["crr_american"]:
        assert close(orc.orc_crr_binomial_american(*row[:8]), row[8], 1e-12)
    # tests/analytic_test.cpp:112 textbook BSM value
    assert abs(orc.orc_bsm(100, 100, .05, 0, .2, 1, 0) - 10.450583572185565) < 1e-12


def test_planted_mistake_is_caught(orc, golden):
    """A restatement error must not pass: perturb one oracle input, expect a miss."""
    case = golden["mc"][0]
    o = O.options(chunk_count=golden["chunk_count"])
    a = list(case["args"])
    r = orc.orc_mc_european(a[0] * (1 + 1e-9), *a[1:9], C.byref(o))
    assert not close(r.price, case["price"])
    assert math.isfinite(r.price)
