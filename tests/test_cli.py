"""The JSON CLI drop-in (derivative-pricing_gb300/cpp/mcd_gpu_cli.cpp) against
the reference's own CLI (apps/mcd_cli/main.cpp).

The fixture tests/golden/cli_responses.json holds the reference CLI's answers
(make_cli_golden.py).  Bars: same exit code, same response keys in the same
order, every number equal to the printed precision (%.10g, so 1e-9
relative) except timings; malformed requests give the same error text.
Requests that need no GPU (forward, binomial trees, the semi-analytic
Heston price, validation errors) run on the CPU; the rest are GPU tests.
"""
from __future__ import annotations

import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "derivative-pricing_gb300", "build", "mcd_gpu_cli")
TIMING = {"elapsed_seconds", "paths_per_second", "note"}


def _cases():
    with open(os.path.join(ROOT, "tests", "golden", "cli_responses.json")) as f:
        return json.load(f)["cases"]


CASES = _cases()
CPU_ONLY = [c for c in CASES if c["exit_code"] != 0 or c["request"]["product"] in ("forward", "binomial_european",
                                                                                    "binomial_american")
            or c["request"].get("request") == "semi_analytic"]
GPU = [c for c in CASES if c not in CPU_ONLY]


@pytest.fixture(scope="module", autouse=True)
def _built():
    import build as B  # derivative-pricing_gb300/build.py (incremental: a no-op when up to date)
    B.build()


def run(req: dict):
    p = subprocess.run([CLI], input=json.dumps(req), capture_output=True, text=True, timeout=300)
    return p.returncode, json.loads(p.stdout)


def check(case):
    rc, got = run(case["request"])
    want = case["response"]
    assert rc == case["exit_code"], (case["request"], got)
    assert list(got.keys()) == list(want.keys()), (case["request"], got, want)
    for k, v in want.items():
        if k in TIMING:
            continue
        if isinstance(v, (int, float)) and not isinstance(v, bool):
            assert abs(got[k] - v) <= 1e-9 * abs(v) + 1e-12, (case["request"], k, got[k], v)
        else:
            assert got[k] == v, (case["request"], k, got[k], v)


def _id(c):
    r = c["request"]
    return f"{r.get('product')}-{r.get('request', 'price')}-{r.get('type', '')}"


@pytest.mark.parametrize("case", CPU_ONLY, ids=_id)
def test_cli_cpu_requests_match_reference(case):
    check(case)


@pytest.mark.gpu
@pytest.mark.parametrize("case", GPU, ids=_id)
def test_cli_gpu_requests_match_reference(case):
    check(case)


@pytest.mark.gpu
def test_cli_batch_matches_single_requests():
    base = dict(type="call", spot=100.0, rate=0.03, carry_yield=0.0, time=1.0, seed=9, path_count=20000,
                monitoring_points=24, strike_style="fixed", average_style="arithmetic")
    strikes = [90.0, 100.0, 110.0]
    vols = [0.15, 0.25, 0.35]
    rc, got = run(dict(base, request="batch", product="asian", strike=strikes, vol=vols))
    assert rc == 0, got
    assert got["count"] == 3
    for i, (k, v) in enumerate(zip(strikes, vols)):
        rc, one = run(dict(base, product="asian", strike=k, vol=v))
        assert rc == 0
        assert got["price"][i] == one["price"] and got["standard_error"][i] == one["standard_error"]
    rc, g = run(dict(base, request="batch_greeks", product="asian", strike=strikes, vol=vols, precision="fp32"))
    assert rc == 0, g
    assert len(g["fd_delta"]) == 3 and g["lr_theta"] == [None, None, None]
    assert all(0.0 < d < 1.0 for d in g["pathwise_delta"])


def test_cli_rejects_malformed_json():
    for text in ("", "{", "[1,2]", '{"product": "forward", "spot": }', '{"a":1} trailing'):
        p = subprocess.run([CLI], input=text, capture_output=True, text=True, timeout=60)
        assert p.returncode == 1 and "error" in json.loads(p.stdout), text
