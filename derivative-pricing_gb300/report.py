"""Validation-report sweeps on the GPU.

The reference regenerates the data-driven part of its validation report from a live
run (tools/generate_report.py:138-330): a table of no-arbitrage invariants of the
closed forms, the standard error of the European price against the path count, the
variance-reduction factors of antithetic sampling and the Asian control variate, the
error of finite-difference delta and gamma against the bump size, and a thread-scaling
curve -- each Monte Carlo point one pricer call.  Here every Monte Carlo sweep is ONE
batch launch of the path engine (``mcd_price_batch``): the points of a sweep are
contracts of one batch, so a sweep costs one graph launch, and because draws are keyed
on (seed, path, step) alone, every point equals the single pricer call bit for bit.
The scaling curve becomes the GPU's: throughput against the work in one launch.

    python derivative-pricing_gb300/report.py [--out report.md] [--json report.json]
        [--update docs/validation-report.md] [--precision fp64|fp32] [--quick]

``--update`` rewrites the block between ``<!-- BEGIN GENERATED -->`` and
``<!-- END GENERATED -->`` of an existing document, as the reference's generator does.
"""
from __future__ import annotations

import argparse
import datetime
import json
import math
import os
import sys
import time

import numpy as np

sys.path.insert(0, os.path.dirname(os.path.abspath(__file__)))
import mcd_gpu as G  # noqa: E402

BEGIN_MARKER = "<!-- BEGIN GENERATED -->"
END_MARKER = "<!-- END GENERATED -->"
TOL = 1e-9


def contract(product, spot, strike, rate, carry_yield, vol, time_, type_, path_count, seed, **kw):
    """One mcd_contract record (numpy, CONTRACT_DTYPE)."""
    c = G.contracts(1)
    c["product"] = product
    c["spot"], c["strike"], c["rate"], c["carry_yield"], c["vol"], c["time"] = (
        spot, strike, rate, carry_yield, vol, time_)
    c["type"] = type_
    c["path_count"] = path_count
    c["seed"] = seed
    for k, v in kw.items():
        c[k] = v
    return c


def batch(records):
    return np.concatenate(records)


# -- 1. invariants of the closed forms (host code, no GPU) ----------------------------------

def cfa_invariants():
    """(module, invariant, passed, deviation) rows: cost of carry, forward values,
    put-call (forward) parity, binomial risk neutrality and convergence, no-arbitrage
    bounds and monotonicity in spot -- the checks of the reference's report table."""
    rows = []
    C, P = G.CALL, G.PUT
    s, r, q, t = 100.0, 0.04, 0.015, 1.5
    dev = abs(G.forward_price(s, r, q, t) - s * math.exp((r - q) * t))
    rows.append(("LM4", "Cost of carry", dev < TOL, dev))
    f0 = G.forward_price(100.0, 0.03, 0.01, 1.0)
    dev = abs(G.forward_value(f0, f0, 0.03, 1.0))
    rows.append(("LM5", "Forward value at initiation is zero", dev < TOL, dev))
    dev = abs(G.forward_value(112.0, 105.0, 0.03, 0.4) - 7.0 * math.exp(-0.03 * 0.4))
    rows.append(("LM5", "Forward value during life", dev < TOL, dev))
    call = G.black_scholes_merton(100, 100, 0.04, 0.01, 0.25, 1.0, C)
    put = G.black_scholes_merton(100, 100, 0.04, 0.01, 0.25, 1.0, P)
    lhs = call + 100 * math.exp(-0.04)
    dev = abs(lhs - (put + 100 * math.exp(-0.01)))
    rows.append(("LM9", "Put-call parity", dev < 1e-12, dev))
    dev = abs(lhs - (put + G.forward_price(100, 0.04, 0.01, 1.0) * math.exp(-0.04)))
    rows.append(("LM9", "Put-call forward parity", dev < 1e-12, dev))
    b = G.crr_binomial(100, 100, 0.05, 0.01, 0.25, 1.0, 1, C)
    p_expected = (math.exp(0.04) - b.down_factor) / (b.up_factor - b.down_factor)
    dev = abs(b.risk_neutral_probability - p_expected)
    rows.append(("LM10", "Binomial risk-neutrality", dev < TOL and 0 < b.risk_neutral_probability < 1, dev))
    bsm = G.black_scholes_merton(100, 100, 0.05, 0.02, 0.2, 1.0, C)
    errs = [abs(G.crr_binomial(100, 100, 0.05, 0.02, 0.2, 1.0, n, C).price - bsm) for n in (10, 50, 250, 1000, 5000)]
    ok = all(b2 < a2 for a2, b2 in zip(errs, errs[1:])) and errs[-1] < 0.01
    rows.append(("LM10", "Binomial converges to BSM (monotonically, error<0.01 at n=5000)", ok, errs[-1]))
    ok = True
    for s2 in (50.0, 100.0, 150.0):
        for k2 in (80.0, 100.0, 120.0):
            c2 = G.black_scholes_merton(s2, k2, 0.04, 0.015, 0.3, 1.0, C)
            lo = max(s2 * math.exp(-0.015) - k2 * math.exp(-0.04), 0.0)
            ok = ok and lo - TOL <= c2 <= s2 * math.exp(-0.015) + TOL
    rows.append(("LM4/LM8", "No-arbitrage bounds", ok, 0.0))
    prices = [G.black_scholes_merton(50.0 + 5.0 * i, 100, 0.04, 0.01, 0.25, 1.0, C) for i in range(21)]
    ok = all(b2 >= a2 - TOL for a2, b2 in zip(prices, prices[1:]))
    rows.append(("LM8", "Monotonicity in spot", ok, 0.0))
    return rows


# -- 2. convergence: standard error against path count, one launch ------------------------

def convergence(eng, counts=(10**3, 10**4, 10**5, 10**6, 10**7, 10**8), seed=123, precision="fp64"):
    recs = [contract(G.EUROPEAN, 100, 100, 0.05, 0.0, 0.2, 1.0, G.CALL, n, seed) for n in counts]
    out = eng.price_batch(batch(recs), precision)
    points = [(int(n), float(se)) for n, se in zip(counts, out["standard_error"])]
    xs = np.log10([p[0] for p in points])
    ys = np.log10([p[1] for p in points])
    slope = float(np.polyfit(xs, ys, 1)[0])
    return {"points": points, "slope": slope, "prices": [float(x) for x in out["price"]]}


# -- 3. variance-reduction factors, one launch ------------------------------------------------

def variance_reduction(eng, n=200_000, seed=7, precision="fp64"):
    """plain / reduced variance for: European antithetic, arithmetic Asian with the
    geometric control variate (the reference's two rows), and arithmetic Asian
    antithetic."""
    base = dict(spot=100, strike=100, rate=0.05, carry_yield=0.0, vol=0.2, time_=1.0, type_=G.CALL,
                path_count=n, seed=seed)
    asian = dict(strike_style=G.FIXED, average_style=G.ARITHMETIC, monitoring_points=12)
    recs = [contract(G.EUROPEAN, **base),
            contract(G.EUROPEAN, **base, antithetic=1),
            contract(G.ASIAN, **base, **asian),
            contract(G.ASIAN, **base, **asian, control_variate=1),
            contract(G.ASIAN, **base, **asian, antithetic=1)]
    out = eng.price_batch(batch(recs), precision)
    se = out["standard_error"]
    rows = [("European", "antithetic", float(se[0] ** 2 / se[1] ** 2)),
            ("Arithmetic Asian", "control variate (geometric Asian)", float(se[2] ** 2 / se[3] ** 2)),
            ("Arithmetic Asian", "antithetic", float(se[2] ** 2 / se[4] ** 2))]
    return {"rows": rows, "prices": [float(x) for x in out["price"]]}


# -- 4. finite-difference bump-size sweep, one launch ----------------------------------------

def bump_sweep(eng, n=200_000, seed=777, precision="fp64"):
    s, k, r, q, v, t = 100.0, 100.0, 0.05, 0.0, 0.20, 1.0
    h6 = s * 1e-6
    true_delta = (G.black_scholes_merton(s + h6, k, r, q, v, t, G.CALL) -
                  G.black_scholes_merton(s - h6, k, r, q, v, t, G.CALL)) / (2 * h6)
    h4 = s * 1e-4
    true_gamma = (G.black_scholes_merton(s + h4, k, r, q, v, t, G.CALL) -
                  2 * G.black_scholes_merton(s, k, r, q, v, t, G.CALL) +
                  G.black_scholes_merton(s - h4, k, r, q, v, t, G.CALL)) / (h4 * h4)
    fracs = [1e-6 * 10 ** (0.5 * i) for i in range(12)]  # 1e-6 .. 0.32, half-decade steps (h < S)
    recs = [contract(G.EUROPEAN, s, k, r, q, v, t, G.CALL, n, seed)]
    for f in fracs:
        recs.append(contract(G.EUROPEAN, s + s * f, k, r, q, v, t, G.CALL, n, seed))
        recs.append(contract(G.EUROPEAN, s - s * f, k, r, q, v, t, G.CALL, n, seed))
    out = eng.price_batch(batch(recs), precision)["price"]
    v0 = out[0]
    delta_pts, gamma_pts = [], []
    for i, f in enumerate(fracs):
        h = s * f
        up, dn = out[1 + 2 * i], out[2 + 2 * i]
        d_err = abs((up - dn) / (2 * h) - true_delta)
        g_err = abs((up - 2 * v0 + dn) / (h * h) - true_gamma)
        if d_err > 0 and g_err > 0:
            delta_pts.append((f, float(d_err)))
            gamma_pts.append((f, float(g_err)))
    best = min(gamma_pts, key=lambda p: p[1])
    return {"delta": delta_pts, "gamma": gamma_pts, "best_gamma": best,
            "true_delta": true_delta, "true_gamma": true_gamma}


# -- 5. scaling: throughput against the work in one launch -----------------------------------

def scaling(eng, counts=(10**4, 10**5, 10**6, 10**7, 10**8, 10**9), precision="fp32", reps=3):
    """Paths/s of one European contract against its path count (the GPU fills as the
    launch grows), wall clock of the pricer call, best of reps after a warm-up."""
    points = []
    for n in counts:
        args = (100, 100, 0.05, 0.0, 0.2, 1.0, G.CALL, int(n), 42)
        eng.monte_carlo_european(*args, precision=precision)
        best = float("inf")
        for _ in range(reps):
            t0 = time.perf_counter()
            eng.monte_carlo_european(*args, precision=precision)
            best = min(best, time.perf_counter() - t0)
        points.append((int(n), n / best))
    return {"points": points, "peak_paths_per_second": max(p[1] for p in points)}


# -- assembly ---------------------------------------------------------------------------------

def run(eng, quick=False, precision="fp64"):
    t0 = time.perf_counter()
    res = {"generated": datetime.datetime.now(datetime.timezone.utc).strftime("%Y-%m-%d %H:%M UTC"),
           "precision": precision,
           "invariants": cfa_invariants(),
           "convergence": convergence(eng, counts=(10**3, 10**4, 10**5, 10**6) if quick else
                                      (10**3, 10**4, 10**5, 10**6, 10**7, 10**8), precision=precision),
           "variance_reduction": variance_reduction(eng, n=50_000 if quick else 200_000, precision=precision),
           "bump_sweep": bump_sweep(eng, n=50_000 if quick else 200_000, precision=precision),
           "scaling": scaling(eng, counts=(10**4, 10**5, 10**6) if quick else
                              (10**4, 10**5, 10**6, 10**7, 10**8, 10**9))}
    res["elapsed_seconds"] = time.perf_counter() - t0
    return res


def markdown(res):
    out = [BEGIN_MARKER, "",
           f"_Generated by `python derivative-pricing_gb300/report.py` on {res['generated']} "
           f"({res['precision'].upper()} paths on the GPU, {res['elapsed_seconds']:.2f} s for every sweep)._", "",
           "### Invariants of the closed forms", "",
           "| Module | Invariant | Result | Measured deviation |", "|---|---|---|---|"]
    for module, name, ok, dev in res["invariants"]:
        out.append(f"| {module} | {name} | {'PASS' if ok else '**FAIL**'} | {dev:.3e} |")
    conv = res["convergence"]
    out += ["", "### Convergence: standard error vs. path count (one batch launch)", "",
            "| Path count | Standard error |", "|---:|---:|"]
    out += [f"| {n:,} | {se:.6f} |" for n, se in conv["points"]]
    out += ["", f"Fitted log-log slope: **{conv['slope']:.4f}** (theory: -0.5).", "",
            "### Variance-reduction factors (one batch launch)", "",
            "| Product | Technique | Variance-reduction factor |", "|---|---|---:|"]
    out += [f"| {p} | {tech} | {f:.2f}x |" for p, tech, f in res["variance_reduction"]["rows"]]
    bs = res["bump_sweep"]
    out += ["", "### Bump-size sweep for finite-difference Greeks (one batch launch)", "",
            "| h/S | delta error | gamma error |", "|---:|---:|---:|"]
    out += [f"| {f:.2e} | {d:.3e} | {g:.3e} |" for (f, d), (_, g) in zip(bs["delta"], bs["gamma"])]
    out += ["", f"Gamma-error minimum: h/S = {bs['best_gamma'][0]:.3e}, error = {bs['best_gamma'][1]:.3e}.", "",
            "### GPU scaling: throughput vs. paths in one launch (European, FP32)", "",
            "| Paths | Paths/s |", "|---:|---:|"]
    out += [f"| {n:,} | {pps:.3e} |" for n, pps in res["scaling"]["points"]]
    out += ["", END_MARKER]
    return "\n".join(out)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("--out", help="write the generated block to this file")
    ap.add_argument("--json", help="write the raw results as JSON")
    ap.add_argument("--update", help="replace the generated block of an existing document")
    ap.add_argument("--precision", default="fp64", choices=("fp64", "fp32"))
    ap.add_argument("--quick", action="store_true", help="small sweeps (seconds)")
    ap.add_argument("--device", type=int, default=int(os.environ.get("MCD_GPU_DEVICE", "0")))
    a = ap.parse_args(argv)
    with G.Engine(a.device) as eng:
        res = run(eng, quick=a.quick, precision=a.precision)
    block = markdown(res)
    if a.json:
        with open(a.json, "w") as f:
            json.dump(res, f, indent=1)
    if a.update:
        text = open(a.update).read()
        if BEGIN_MARKER not in text or END_MARKER not in text:
            raise SystemExit(f"{a.update} has no {BEGIN_MARKER} / {END_MARKER} block")
        text = text[:text.index(BEGIN_MARKER)] + block + text[text.index(END_MARKER) + len(END_MARKER):]
        with open(a.update, "w") as f:
            f.write(text)
    if a.out:
        with open(a.out, "w") as f:
            f.write(block + "\n")
    if not (a.out or a.update):
        print(block)
    return 0


if __name__ == "__main__":
    sys.exit(main())
