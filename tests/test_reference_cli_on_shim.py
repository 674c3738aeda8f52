"""The reference's own JSON CLI (apps/mcd_cli/main.cpp), compiled unchanged
against the GPU shim.

derivative-pricing_gb300/cpp/compat holds forwarding headers: each of the
reference's mcd/pricers/*, mcd/greeks/*, mcd/models/heston, mcd/core/types,
mcd/core/sobol and mcd/core/rng_simd headers resolves to cpp/mcd_shim.hpp, so a
reference caller
builds without an edit and links libmcd_shim.so (the GPU engine) instead of
libmcd_core.a.  Only the CLI's JSON reader (src/core/json.cpp) still comes from
the reference.  The recipe is oracle/Makefile's ``refcli-on-shim`` target; it
needs the reference's sources, so the test is skipped where they are absent.

Bars: the requests the shim answers on the host (forward prices, lattices, the
semi-analytic Heston price, validation errors) give the reference CLI's own
responses (tests/golden/cli_responses.json) to its printed precision.
"""
from __future__ import annotations

import json
import os
import subprocess

import pytest

import test_cli as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
CLI = os.path.join(ORACLE, "_ref", "mcd_cli_on_shim")


@pytest.fixture(scope="module")
def cli():
    if subprocess.run(["make", "-s", "-C", ORACLE, "has-ref"], capture_output=True).returncode != 0:
        pytest.skip("the reference's sources are not on this machine")
    import build as B
    B.build()
    r = subprocess.run(["make", "-s", "-C", ORACLE, "refcli-on-shim"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stdout + r.stderr)
    return CLI


@pytest.mark.parametrize("case", T.CPU_ONLY, ids=T._id)
def test_reference_cli_unchanged_on_the_shim(cli, case):
    p = subprocess.run([cli], input=json.dumps(case["request"]), capture_output=True, text=True, timeout=120)
    got = json.loads(p.stdout)
    want = case["response"]
    assert p.returncode == case["exit_code"], (case["request"], got)
    assert list(got.keys()) == list(want.keys()), (case["request"], got, want)
    for k, v in want.items():
        if k in T.TIMING:
            continue
        if isinstance(v, (int, float)) and not isinstance(v, bool):
            assert abs(got[k] - v) <= 1e-9 * abs(v) + 1e-12, (case["request"], k, got[k], v)
        else:
            assert got[k] == v, (case["request"], k, got[k], v)


@pytest.mark.gpu
@pytest.mark.parametrize("case", T.GPU, ids=T._id)
def test_reference_cli_unchanged_on_the_shim_gpu_requests(cli, case):
    """The Monte Carlo requests through the same binary (GPU, FP64 by
    default: the reference's arithmetic)."""
    test_reference_cli_unchanged_on_the_shim(cli, case)
