"""Generate tests/golden/reference_vectors.json from the reference itself.

Runs the reference library compiled from its own sources (oracle/Makefile,
target ``ref`` -> oracle/_ref/libmcd_ref.so) on small, fixed cases and records
full-precision outputs.  The reference source tree is only needed to build that
library; the committed fixture is what the tests read (on any machine).

Usage:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import ctypes as C
import json
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import oracle as O  # noqa: E402


def main() -> None:
    O.build()
    r = O.load_ref()
    if r is None:
        raise SystemExit("reference library was not built (reference sources missing)")
    chunks = int(r.ref_logical_chunk_count())
    out = {"chunk_count": chunks, "source": "reference compiled from source via oracle/Makefile"}

    # Philox KATs (the reference's own vectors, tests/rng_test.cpp:17-39).
    kats = [
        ([0, 0, 0, 0], [0, 0]),
        ([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2),
        ([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]),
    ]
    rows = []
    for ctr, key in kats:
        o = (C.c_uint32 * 4)()
        r.ref_philox((C.c_uint32 * 4)(*ctr), (C.c_uint32 * 2)(*key), o)
        rows.append({"counter": ctr, "key": key, "out": list(o)})
    out["philox"] = rows

    draws = []
    for seed in (0, 42, 2**40 + 3):
        for path in (0, 1, 4095, 4096, 2**32 + 17):
            for d in (0, 1, 251):
                draws.append([seed, path, d, r.ref_normal_variate(seed, path, d),
                              r.ref_uniform_variate(seed, path, d)])
    out["draws"] = draws
    us = [1e-9, 1e-6, 0.001, 0.02, 0.02425, 0.03, 0.2, 0.5, 0.7, 0.97575, 0.99, 1 - 1e-7]
    out["inv_normal_cdf"] = [[u, r.ref_inv_normal_cdf(u)] for u in us]

    res = O.dbuf(3)
    mc = []

    def add(kind, args, f):
        f(res)
        mc.append({"kind": kind, "args": args, "price": res[0], "se": res[1],
                   "paths": int(res[2])})

    # The headline single-contract case: S0=K=100, r=.05, q=0, sigma=.2, T=1, 1e6 paths, seed 42.
    add("european", [100, 100, .05, 0, .2, 1, 0, 10**6, 42, 0],
        lambda o: r.ref_mc_european(100, 100, .05, 0, .2, 1, 0, 10**6, 42, 0, 1, o))
    add("european", [105, 100, .03, .01, .3, .75, 1, 20003, 7, 1],
        lambda o: r.ref_mc_european(105, 100, .03, .01, .3, .75, 1, 20003, 7, 1, 1, o))
    for style in (0, 1):
        add("digital", [100, 95, .05, .01, .25, 1, 0, style, 1.5, 20003, 9, 0],
            lambda o, s=style: r.ref_mc_digital(100, 95, .05, .01, .25, 1, 0, s, 1.5, 20003, 9, 0, 1, o))
    for ss in (0, 1):
        for av in (0, 1):
            for ty in (0, 1):
                add("asian", [100, 100, .05, 0, .3, 1, ty, ss, av, 12, 20003, 5, 0, 0],
                    lambda o, a=(ty, ss, av): r.ref_mc_asian(100, 100, .05, 0, .3, 1, a[0], a[1], a[2],
                                                             12, 20003, 5, 0, 0, 1, o))
    add("asian", [100, 100, .05, 0, .3, 1, 0, 0, 0, 12, 20003, 5, 0, 1],
        lambda o: r.ref_mc_asian(100, 100, .05, 0, .3, 1, 0, 0, 0, 12, 20003, 5, 0, 1, 1, o))
    add("asian", [100, 100, .05, 0, .3, 1, 1, 0, 0, 24, 20003, 5, 1, 0],
        lambda o: r.ref_mc_asian(100, 100, .05, 0, .3, 1, 1, 0, 0, 24, 20003, 5, 1, 0, 1, o))
    for d in (0, 1):
        for k in (0, 1):
            for ty in (0, 1):
                for bb in (0, 1):
                    h = 120.0 if d == 0 else 85.0
                    add("barrier", [100, 100, h, .05, 0, .25, 1, ty, d, k, .5, 20, 20003, 3, 0, bb],
                        lambda o, a=(h, ty, d, k, bb): r.ref_mc_barrier(
                            100, 100, a[0], .05, 0, .25, 1, a[1], a[2], a[3], .5, 20, 20003, 3, 0,
                            a[4], 1, o))
    for ss in (0, 1):
        for ty in (0, 1):
            add("lookback", [100, 100, .05, 0, .25, 1, ty, ss, 30, 20003, 3, 0],
                lambda o, a=(ty, ss): r.ref_mc_lookback(100, 100, .05, 0, .25, 1, a[0], a[1], 30,
                                                        20003, 3, 0, 1, o))
    out["mc"] = mc

    # Longstaff-Schwartz, 50 dates.
    lsm = []
    for (s, k, rr, q, v, t, ty, n, paths) in [(36, 40, .06, 0, .2, 1, 1, 50, 1 << 14),
                                              (44, 40, .06, 0, .4, 2, 1, 50, 1 << 13),
                                              (100, 100, .05, .03, .3, .5, 0, 25, 1 << 13)]:
        ro = O.dbuf(2)
        co = O.dbuf((n + 1) * 4)
        ho = (C.c_uint8 * (n + 1))()
        inc = C.c_int(0)
        r.ref_lsm_american(s, k, rr, q, v, t, ty, n, paths, 42, ro, co, ho, C.byref(inc))
        lsm.append({"args": [s, k, rr, q, v, t, ty, n, paths, 42], "price": ro[0], "se": ro[1],
                    "coefficients": list(co), "has": list(ho), "inception": inc.value})
    out["lsm"] = lsm

    heston = []
    lewis = [100, .01, .02, .04, 4, .25, 1, -.5, 1]
    p9 = O.dbuf(9)
    for i, x in enumerate(lewis):
        p9[i] = x
    for k in (80, 100, 120):
        for ty in (0, 1):
            r.ref_heston_qe(p9, k, ty, 50, 4000, 11, res)
            heston.append({"params": lewis, "strike": k, "type": ty, "steps": 50, "paths": 4000,
                           "seed": 11, "price": res[0], "se": res[1],
                           "semi_analytic": r.ref_heston_semi_analytic(p9, k, ty)})
    out["heston"] = heston

    out["sobol"] = {str(d): [r.ref_sobol_point(d, i) for i in range(70)] for d in range(7)}
    out["qmc_european"] = [[100, 100, .05, 0, .2, 1, 0, 100000,
                            r.ref_qmc_european(100, 100, .05, 0, .2, 1, 0, 100000)]]
    out["qmc_asian"] = [[100, 100, .05, 0, .2, 1, 0, ss, n, 20000,
                         r.ref_qmc_asian(100, 100, .05, 0, .2, 1, 0, ss, n, 20000)]
                        for n in range(1, 8) for ss in (0, 1)]

    bumps = O.dbuf(4)
    r.ref_default_bumps(100, .2, 1, bumps)
    fd = O.dbuf(5)
    r.ref_fd_european(100, 100, .05, 0, .2, 1, 0, 100000, 42, bumps, fd)
    out["fd_european"] = {"args": [100, 100, .05, 0, .2, 1, 0, 100000, 42],
                          "bumps": list(bumps), "greeks": list(fd)}
    g = O.dbuf(10)
    r.ref_lr_european(100, 100, .05, 0, .2, 1, 0, 50000, 42, g)
    lr = {"european": {"args": [100, 100, .05, 0, .2, 1, 0, 50000, 42], "out": list(g)}}
    r.ref_lr_digital(100, 100, .05, 0, .2, 1, 0, 0, 1.0, 50000, 42, g)
    lr["digital"] = {"args": [100, 100, .05, 0, .2, 1, 0, 0, 1.0, 50000, 42], "out": list(g)}
    r.ref_lr_barrier(100, 100, 120, .05, 0, .2, 1, 0, 0, 1, 0, 20, 20000, 42, g)
    lr["barrier"] = {"args": [100, 100, 120, .05, 0, .2, 1, 0, 0, 1, 0, 20, 20000, 42],
                     "out": list(g)[:8]}
    out["lr"] = lr
    pw = O.dbuf(6)
    r.ref_pathwise_european(100, 100, .05, 0, .2, 1, 0, 50000, 42, pw)
    pwd = {"european": {"args": [100, 100, .05, 0, .2, 1, 0, 50000, 42], "out": list(pw)}}
    for ss in (0, 1):
        for av in (0, 1):
            r.ref_pathwise_asian(100, 100, .05, 0, .2, 1, 1, ss, av, 12, 20000, 42, pw)
            pwd[f"asian_{ss}{av}"] = {"args": [100, 100, .05, 0, .2, 1, 1, ss, av, 12, 20000, 42],
                                      "out": list(pw)}
    out["pathwise"] = pwd

    D = C.c_double
    for name, res_t, args in (("ref_black76", D, [D] * 5 + [C.c_int]),
                              ("ref_forward_price", D, [D] * 4), ("ref_forward_value", D, [D] * 4),
                              ("ref_futures_mtm", D, [D] * 2),
                              ("ref_crr_european", None, [D] * 6 + [C.c_int, C.c_int, C.POINTER(D)])):
        getattr(r, name).restype = res_t
        getattr(r, name).argtypes = args
    crr4 = (D * 4)()
    crr_eu = []
    for args in ((100, 100, .05, 0, .2, 1, 500, 0), (36, 40, .06, .01, .3, 2, 301, 1)):
        r.ref_crr_european(*args, crr4)
        crr_eu.append(list(args) + list(crr4))
    rr = []
    for ty in (0, 1):
        for d in (0, 1):
            for kn in (0, 1):
                for k, h in ((100, 120), (100, 80), (110, 105), (90, 95)):
                    if (d == 0 and h <= 100) or (d == 1 and h >= 100):
                        continue
                    args = [100, k, h, .05, .01, .25, 1, ty, d, kn, 1.5]
                    rr.append(args + [r.ref_reiner_rubinstein(*args)])
    p9 = (D * 9)(100, .03, 0, .04, 1.5, .05, .6, -.7, 1)
    out["analytic"] = {
        "bsm": [[100, 100, .05, 0, .2, 1, 0, r.ref_bsm(100, 100, .05, 0, .2, 1, 0)],
                [90, 100, .03, .02, .35, 2, 1, r.ref_bsm(90, 100, .03, .02, .35, 2, 1)]],
        "kemna_vorst": [[100, 95, .05, .01, .2, 1, 1, r.ref_kemna_vorst(100, 95, .05, .01, .2, 1, 1)],
                        [100, 105, .05, .0, .3, 1.5, 0, r.ref_kemna_vorst(100, 105, .05, 0, .3, 1.5, 0)]],
        "crr_american": [[36, 40, .06, 0, .2, 1, 500, 1,
                          r.ref_crr_american(36, 40, .06, 0, .2, 1, 500, 1)]],
        "crr_european": crr_eu,
        "black76": [[105, 100, .04, .25, 1.5, ty, r.ref_black76(105, 100, .04, .25, 1.5, ty)] for ty in (0, 1)],
        "reiner_rubinstein": rr,
        "lookback_fixed": [[100, k, .05, .01, .3, 1, ty, r.ref_lookback_fixed(100, k, .05, .01, .3, 1, ty)]
                           for k in (90, 100, 110) for ty in (0, 1)],
        "lookback_floating": [[100, .05, .01, .3, 1, ty, r.ref_lookback_floating(100, .05, .01, .3, 1, ty)]
                              for ty in (0, 1)],
        "digital": [[100, 95, .05, .01, .2, 1, ty, st, 2.0, r.ref_digital_analytic(100, 95, .05, .01, .2, 1, ty, st, 2.0)]
                    for ty in (0, 1) for st in (0, 1)],
        "forward_price": [[100, .05, .01, 2, r.ref_forward_price(100, .05, .01, 2)]],
        "forward_value": [[110, 104, .05, .5, r.ref_forward_value(110, 104, .05, .5)]],
        "futures_mtm": [[101.5, 100.25, r.ref_futures_mtm(101.5, 100.25)]],
        "heston_semi_analytic": [[list(p9), k, ty, r.ref_heston_semi_analytic(p9, k, ty)]
                                 for k in (90, 105) for ty in (0, 1)],
    }
    path = os.path.join(HERE, "reference_vectors.json")
    with open(path, "w") as f:
        json.dump(out, f, indent=0)
    print("wrote", path, os.path.getsize(path), "bytes")


if __name__ == "__main__":
    main()
