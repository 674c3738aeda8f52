"""Generates cli_responses.json: the reference's own JSON CLI (apps/mcd_cli/main.cpp,
built from its sources by `make -C oracle refcli`) answering a fixed set of
requests that covers every product and request kind of its schema, plus
malformed requests.  Run in a checkout that has the reference sources; the
fixture is committed and the tests compare the GPU CLI against it.

    make -C oracle refcli && python tests/golden/make_cli_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_CLI = os.path.join(HERE, "..", "..", "oracle", "_ref", "mcd_cli_ref")

BASE = dict(spot=100, strike=100, rate=0.05, carry_yield=0.01, vol=0.2, time=1, type="call")
REQUESTS = [
    dict(product="forward", spot=100, rate=0.05, carry_yield=0.01, time=2),
    dict(BASE, product="binomial_european", steps=500),
    dict(BASE, product="binomial_american", type="put", steps=800),
    dict(BASE, product="european", path_count=50000, seed=42),
    dict(BASE, product="european", type="put", path_count=30000, seed=7),
    dict(BASE, product="european", request="greeks", path_count=20000, seed=42),
    dict(BASE, product="european", request="lr_greeks", path_count=20000, seed=3),
    dict(BASE, product="european", request="pathwise_greeks", path_count=20000, seed=5),
    dict(BASE, product="european", request="qmc_sobol", path_count=40000),
    dict(BASE, product="digital", digital_style="cash_or_nothing", cash_amount=2.5, path_count=30000, seed=11),
    dict(BASE, product="digital", type="put", digital_style="asset_or_nothing", request="lr_greeks",
         path_count=20000, seed=12),
    dict(BASE, product="asian", strike_style="fixed", average_style="arithmetic", monitoring_points=12,
         path_count=20000, seed=21),
    dict(BASE, product="asian", type="put", strike_style="floating", average_style="geometric",
         monitoring_points=9, path_count=20000, seed=22),
    dict(BASE, product="asian", strike_style="fixed", average_style="arithmetic", monitoring_points=5,
         request="qmc_sobol", path_count=16384),
    dict(BASE, product="asian", strike_style="floating", average_style="arithmetic", monitoring_points=12,
         request="pathwise_greeks", path_count=20000, seed=23),
    dict(BASE, product="barrier", barrier=120, direction="up", knock="out", monitoring_points=24,
         path_count=20000, seed=31),
    dict(BASE, product="barrier", type="put", barrier=85, direction="down", knock="in", rebate=1.5,
         monitoring_points=30, path_count=20000, seed=32),
    dict(BASE, product="barrier", barrier=125, direction="up", knock="out", monitoring_points=20,
         request="lr_greeks", path_count=20000, seed=33),
    dict(BASE, product="lookback", style="fixed", monitoring_points=16, path_count=20000, seed=41),
    dict(BASE, product="lookback", type="put", style="floating", monitoring_points=16, path_count=20000, seed=42),
    dict(BASE, product="american", spot=36, strike=40, rate=0.06, carry_yield=0, type="put", monitoring_points=20,
         path_count=20000, seed=42),
    dict(product="heston", spot=100, strike=105, rate=0.03, carry_yield=0, v0=0.04, kappa=1.5, theta=0.05, xi=0.6,
         rho=-0.7, time=1, type="call", monitoring_points=50, path_count=20000, seed=51),
    dict(product="heston", request="semi_analytic", spot=100, strike=105, rate=0.03, carry_yield=0, v0=0.04,
         kappa=1.5, theta=0.05, xi=0.6, rho=-0.7, time=1, type="put"),
    # malformed requests
    dict(product="european", spot=100),
    dict(BASE, product="european", type="straddle", path_count=100, seed=1),
    dict(BASE, product="european", path_count=100.5, seed=1),
    dict(BASE, product="european", path_count=9007199254740994, seed=1),
    dict(BASE, product="swaption"),
]


def main():
    out = []
    for req in REQUESTS:
        p = subprocess.run([REF_CLI], input=json.dumps(req), capture_output=True, text=True)
        out.append({"request": req, "exit_code": p.returncode, "response": json.loads(p.stdout)})
    with open(os.path.join(HERE, "cli_responses.json"), "w") as f:
        json.dump({"source": "apps/mcd_cli/main.cpp built from the reference sources", "cases": out}, f, indent=1)


if __name__ == "__main__":
    main()
