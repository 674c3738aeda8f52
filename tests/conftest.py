"""Shared fixtures.  GPU tests are marked ``gpu``; everything else runs on CPU.

The oracle (oracle/) is the checker: tests compare the CUDA library, called
through its C ABI, against the oracle and against golden vectors recorded from
the reference itself (tests/golden/reference_vectors.json).
"""
from __future__ import annotations

import json
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "derivative-pricing_gb300")
for p in (ROOT, PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


@pytest.fixture(scope="session")
def golden():
    with open(os.path.join(ROOT, "tests", "golden", "reference_vectors.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def orc():
    import oracle as O
    O.build()
    return O.load()


@pytest.fixture(scope="session")
def gpu_lib():
    import build as B  # derivative-pricing_gb300/build.py
    B.build()
    import mcd_gpu
    return mcd_gpu


@pytest.fixture(scope="session")
def engine(gpu_lib):
    eng = gpu_lib.Engine(0)
    yield eng
    eng.close()
