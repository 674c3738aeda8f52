"""The Lambda-style handler (derivative-pricing_gb300/lambda_handler.py) against the
reference's own Lambda layer (infra/lambda/handler.py over its pybind11 module),
answering the same API Gateway events (tests/golden/lambda_responses.json, made by
tests/golden/make_lambda_golden.py): same routes, status codes, response fields and
error messages; numbers within the FP64 bars of the pricers (the GPU's FP64 path
against the reference's CPU: 1e-12 relative for prices and standard errors, 1e-10 for
likelihood-ratio and pathwise Greeks and the Longstaff-Schwartz price, 1e-6 for
finite-difference Greeks, whose bumps amplify the last bits of the prices).

Requests that need no simulation (closed forms, validation, routes) run on CPU; the
Monte Carlo ones are marked gpu."""
from __future__ import annotations

import json
import math

import pytest

with open(__file__.rsplit("/", 1)[0] + "/golden/lambda_responses.json") as _f:
    CASES = json.load(_f)["cases"]

CPU_ONLY = {"forward", "binomial_european", "binomial_american", "heston_semi_analytic", "cfa_invariants",
            "unknown_route"}


def needs_gpu(case):
    return case["status"] == 200 and case["name"] not in CPU_ONLY


def tolerance(name, key):
    if name == "european_fd_greeks":
        return 1e-6
    if name == "american" or name.endswith(("lr_greeks", "pathwise")) or key.endswith("_se"):
        return 1e-10
    return 1e-12


@pytest.fixture(scope="module")
def handler(gpu_lib):
    import lambda_handler as L
    return L


def check(handler, case):
    r = handler.lambda_handler(case["event"], None)
    assert r["statusCode"] == case["status"], (case["name"], r)
    assert r["headers"]["Content-Type"] == "application/json"
    body = json.loads(r["body"])
    for k in ("elapsed_seconds", "paths_per_second"):
        body.pop(k, None)
    want = case["body"]
    assert list(body) == list(want), (case["name"], list(body), list(want))  # same fields, same order
    for k, v in want.items():
        got = body[k]
        if k == "invariants":
            assert [(x["module"], x["invariant"], x["pass"]) for x in got] == \
                   [(x["module"], x["invariant"], x["pass"]) for x in v]
            for a, b in zip(got, v):
                assert abs(a["deviation"] - b["deviation"]) <= 1e-12
        elif isinstance(v, float) and not isinstance(v, bool):
            tol = tolerance(case["name"], k)
            assert math.isclose(got, v, rel_tol=tol, abs_tol=tol * 1e-2), (case["name"], k, got, v)
        else:
            assert got == v, (case["name"], k, got, v)


@pytest.mark.parametrize("case", [c for c in CASES if not needs_gpu(c)], ids=lambda c: c["name"])
def test_without_simulation(handler, case):
    check(handler, case)


@pytest.mark.gpu
@pytest.mark.parametrize("case", [c for c in CASES if needs_gpu(c)], ids=lambda c: c["name"])
def test_monte_carlo_requests(handler, case):
    check(handler, case)


def test_path_count_cap_is_configurable(handler, monkeypatch):
    body = {"product": "european", "spot": 100, "strike": 100, "rate": 0.05, "carry_yield": 0.0, "vol": 0.2,
            "time": 1.0, "type": "call", "path_count": 2_000_000, "seed": 1}
    monkeypatch.setattr(handler, "MAX_PATH_COUNT", 1_000_000)
    r = handler.lambda_handler({"routeKey": "POST /price", "body": json.dumps(body)}, None)
    assert r["statusCode"] == 400
    assert "must not exceed 1,000,000" in json.loads(r["body"])["error"]
