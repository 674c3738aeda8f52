"""Generates tests/golden/lambda_responses.json: the reference's AWS Lambda request
layer (infra/lambda/handler.py over its pybind11 module `mcd`) answering a fixed set
of API Gateway events -- every product and request kind of POST /price, the
validation failures, GET /cfa-invariants and an unknown route.  Timing fields
(elapsed_seconds, paths_per_second) are dropped.  The GPU handler
(derivative-pricing_gb300/lambda_handler.py) is tested against these answers.

Needs the reference tree and a C++ compiler: the pybind11 module is built from a
copy of the tree in a temporary directory (the tree itself is never written).

    python tests/golden/make_lambda_golden.py --reference <reference checkout>
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "lambda_responses.json")
TIMING = ("elapsed_seconds", "paths_per_second")

BASE = {"spot": 100, "strike": 100, "rate": 0.05, "carry_yield": 0.0, "vol": 0.2, "time": 1.0, "type": "call"}
HESTON = {"spot": 100, "strike": 100, "rate": 0.01, "carry_yield": 0.02, "v0": 0.04, "kappa": 4.0, "theta": 0.25,
          "xi": 1.0, "rho": -0.5, "time": 1.0, "type": "call"}


def requests():
    """(name, event) pairs; bodies are JSON text as API Gateway delivers them."""
    P = []

    def post(name, body):
        P.append((name, {"routeKey": "POST /price", "body": json.dumps(body)}))

    post("forward", {"product": "forward", "spot": 100, "rate": 0.05, "carry_yield": 0.01, "time": 2.0})
    post("binomial_european", dict(BASE, product="binomial_european", steps=500))
    post("binomial_american", dict(BASE, product="binomial_american", type="put", steps=500))
    post("european", dict(BASE, product="european", path_count=100_000, seed=42))
    post("european_antithetic", dict(BASE, product="european", path_count=100_000, seed=42, antithetic=True))
    post("european_fd_greeks", dict(BASE, product="european", request="greeks", path_count=100_000, seed=42))
    post("european_lr_greeks", dict(BASE, product="european", request="lr_greeks", path_count=100_000, seed=7))
    post("european_pathwise", dict(BASE, product="european", request="pathwise_greeks", path_count=100_000, seed=7))
    post("european_qmc", dict(BASE, product="european", request="qmc_sobol", path_count=65_536))
    post("digital", dict(BASE, product="digital", digital_style="cash_or_nothing", cash_amount=2.0,
                         path_count=100_000, seed=5))
    post("digital_lr_greeks", dict(BASE, product="digital", request="lr_greeks", digital_style="asset_or_nothing",
                                   path_count=100_000, seed=5))
    asian = dict(BASE, product="asian", strike_style="fixed", average_style="arithmetic", monitoring_points=12)
    post("asian", dict(asian, path_count=50_000, seed=9))
    post("asian_control_variate", dict(asian, path_count=50_000, seed=9, control_variate=True))
    post("asian_geometric_floating", dict(asian, strike_style="floating", average_style="geometric",
                                          path_count=50_000, seed=9))
    post("asian_qmc", dict(asian, request="qmc_sobol", monitoring_points=6, path_count=32_768))
    post("asian_pathwise", dict(asian, request="pathwise_greeks", path_count=50_000, seed=9))
    barrier = dict(BASE, product="barrier", barrier=120, direction="up", knock="out", rebate=0.5,
                   monitoring_points=20)
    post("barrier", dict(barrier, path_count=50_000, seed=11))
    post("barrier_down_in", dict(barrier, barrier=85, direction="down", knock="in", path_count=50_000, seed=11))
    post("barrier_lr_greeks", dict(barrier, request="lr_greeks", path_count=50_000, seed=11))
    post("lookback_floating", dict(BASE, product="lookback", style="floating", monitoring_points=20,
                                   path_count=50_000, seed=13))
    post("lookback_fixed_put", dict(BASE, product="lookback", style="fixed", type="put", strike=95,
                                    monitoring_points=20, path_count=50_000, seed=13))
    post("american", dict(BASE, product="american", type="put", spot=36, strike=40, rate=0.06,
                          monitoring_points=20, path_count=20_000, seed=3))
    post("heston_semi_analytic", dict(HESTON, product="heston", request="semi_analytic"))
    post("heston_qe", dict(HESTON, product="heston", monitoring_points=20, path_count=20_000, seed=42))
    # validation failures
    post("err_missing_product", {"spot": 100})
    post("err_unknown_product", {"product": "swaption"})
    post("err_missing_field", {"product": "european", "spot": 100})
    post("err_number_type", dict(BASE, product="european", spot="100", path_count=10, seed=1))
    post("err_bad_type", dict(BASE, product="european", type="straddle", path_count=10, seed=1))
    post("err_path_cap", dict(BASE, product="european", path_count=6_000_000, seed=1))
    post("err_count_fraction", dict(BASE, product="european", path_count=1000, seed=1.5))
    post("err_count_negative", dict(BASE, product="european", path_count=-5, seed=1))
    post("err_steps_cap", dict(BASE, product="binomial_european", steps=30_000))
    post("err_steps_int", dict(BASE, product="binomial_european", steps=10.5))
    post("err_direction", dict(barrier, direction="sideways", path_count=10, seed=1))
    post("err_knock", dict(barrier, knock="maybe", path_count=10, seed=1))
    post("err_strike_style", dict(asian, strike_style="mid", path_count=10, seed=1))
    post("err_lookback_style", dict(BASE, product="lookback", style="mid", monitoring_points=5, path_count=10,
                                    seed=1))
    post("err_average_style", dict(asian, average_style="harmonic", path_count=10, seed=1))
    post("err_digital_style", dict(BASE, product="digital", digital_style="coin", path_count=10, seed=1))
    post("err_qmc_geometric", dict(asian, request="qmc_sobol", average_style="geometric", path_count=1024))
    P.append(("err_malformed_json", {"routeKey": "POST /price", "body": "{not json"}))
    P.append(("err_not_object", {"routeKey": "POST /price", "body": "[1, 2]"}))
    P.append(("cfa_invariants", {"routeKey": "GET /cfa-invariants"}))
    P.append(("unknown_route", {"routeKey": "DELETE /price"}))
    return P


def build_module(reference, work):
    tree = os.path.join(work, "tree")
    shutil.copytree(reference, tree, ignore=shutil.ignore_patterns(".git", "build*", "web", "node_modules"))
    subprocess.run([sys.executable, "setup.py", "build_ext", "--inplace"], cwd=tree, check=True,
                   stdout=subprocess.DEVNULL)
    return tree


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", default=os.environ.get("MCD_REFERENCE_ROOT"),
                    required="MCD_REFERENCE_ROOT" not in os.environ,
                    help="the reference's source checkout (or set MCD_REFERENCE_ROOT)")
    a = ap.parse_args()
    with tempfile.TemporaryDirectory() as work:
        tree = build_module(a.reference, work)
        sys.path[:0] = [tree, os.path.join(tree, "infra", "lambda")]
        import handler  # the reference's Lambda entry point, over its own module

        cases = []
        for name, event in requests():
            r = handler.lambda_handler(event, None)
            body = json.loads(r["body"])
            for k in TIMING:
                body.pop(k, None)
            cases.append({"name": name, "event": event, "status": r["statusCode"], "body": body})
    with open(OUT, "w") as f:
        json.dump({"source": "reference infra/lambda/handler.py over its pybind11 module",
                   "cases": cases}, f, indent=1)
    print(f"wrote {OUT}: {len(cases)} cases")


if __name__ == "__main__":
    main()
