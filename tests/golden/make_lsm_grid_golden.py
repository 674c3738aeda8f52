"""Generate tests/golden/lsm_grid_2p20.json from the reference itself.

The American-put grid at full size: S0 in {36,38,40,42,44}, K=40, r=.06, q=0,
sigma in {.2,.4}, T in {1,2}, 50 exercise dates, 2^20 paths, put, seed 42+i in
that order (S0 outermost, T innermost).  Each put is priced by the reference's
monte_carlo_lsm_american (src/pricers/lsm.cpp:62-149) compiled from its own
sources (oracle/Makefile, target ``ref`` -> oracle/_ref/libmcd_ref.so); price,
standard error, inception flag and the per-date Householder coefficients
(src/core/linalg.cpp:7-71) are recorded at full precision.  The first row is
the S0=36, sigma=.2, T=1, seed 42 put (price 4.476383949663612).

The reference prices one put on one thread (about 13-25 s each here); the
puts run in parallel worker processes.

Usage:  python tests/golden/make_lsm_grid_golden.py [--workers 8]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import multiprocessing as mp
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

PATHS = 1 << 20
DATES = 50


def grid():
    rows = []
    for s in (36, 38, 40, 42, 44):
        for v in (0.2, 0.4):
            for t in (1.0, 2.0):
                rows.append([float(s), 40.0, 0.06, 0.0, v, t, 1, DATES, PATHS, 42 + len(rows)])
    return rows


def price_one(args):
    import oracle as O
    r = O.load_ref()
    s, k, rr, q, v, t, ty, n, paths, seed = args
    ro = O.dbuf(2)
    co = O.dbuf((n + 1) * 4)
    ho = (C.c_uint8 * (n + 1))()
    inc = C.c_int(0)
    r.ref_lsm_american(s, k, rr, q, v, t, ty, n, paths, seed, ro, co, ho, C.byref(inc))
    return {"args": args, "price": ro[0], "se": ro[1], "coefficients": list(co), "has": list(ho),
            "inception": inc.value}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--workers", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    import oracle as O
    O.build()
    if O.load_ref() is None:
        raise SystemExit("reference library was not built (reference sources missing)")
    with mp.get_context("spawn").Pool(a.workers) as pool:
        rows = pool.map(price_one, grid())
    out = {"source": "reference monte_carlo_lsm_american compiled from source via oracle/Makefile",
           "paths": PATHS, "dates": DATES, "puts": rows}
    with open(os.path.join(HERE, "lsm_grid_2p20.json"), "w") as f:
        json.dump(out, f, separators=(",", ":"))
    for r in rows:
        print(r["args"][0], r["args"][4], r["args"][5], repr(r["price"]), r["se"])


if __name__ == "__main__":
    main()
