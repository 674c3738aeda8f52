"""Report sweeps (derivative-pricing_gb300/report.py), the GPU form of the reference's
tools/generate_report.py:138-330: the invariants table on CPU; the Monte Carlo sweeps on
the GPU, each one batch launch whose points must equal the single pricer calls bit for
bit, and whose statistics must say what the reference's report says (SE slope -1/2,
variance-reduction factors above 1, a gamma-error minimum at an interior bump size)."""
from __future__ import annotations

import os

import pytest


@pytest.fixture(scope="module")
def report(gpu_lib):
    import report as R
    return R


def test_invariants_all_pass(report):
    rows = report.cfa_invariants()
    assert len(rows) == 9
    failed = [r for r in rows if not r[2]]
    assert not failed, failed


@pytest.mark.gpu
def test_sweeps(report, engine, gpu_lib, tmp_path):
    res = report.run(engine, quick=True, precision="fp64")
    conv = res["convergence"]
    assert -0.6 < conv["slope"] < -0.4
    # each point of the one-launch sweep is the single pricer call, bit for bit
    for (n, se), price in zip(conv["points"], conv["prices"]):
        one = engine.monte_carlo_european(100, 100, 0.05, 0.0, 0.2, 1.0, gpu_lib.CALL, n, 123)
        assert one.price == price and one.standard_error == se
    vr = {(p, t): f for p, t, f in res["variance_reduction"]["rows"]}
    assert vr[("European", "antithetic")] > 1.5
    assert vr[("Arithmetic Asian", "control variate (geometric Asian)")] > 10.0
    cv = engine.monte_carlo_asian(100, 100, 0.05, 0.0, 0.2, 1.0, gpu_lib.CALL, gpu_lib.FIXED,
                                  gpu_lib.ARITHMETIC, 12, 50_000, 7, control_variate=True)
    assert res["variance_reduction"]["prices"][3] == cv.price
    bs = res["bump_sweep"]
    f_best, err_best = bs["best_gamma"]
    assert 1e-3 <= f_best <= 0.3, bs["best_gamma"]
    assert bs["gamma"][0][1] > 100 * err_best  # tiny bumps: cancellation noise dominates
    pts = res["scaling"]["points"]
    assert pts[-1][1] > pts[0][1]  # more paths per launch, higher throughput
    block = report.markdown(res)
    assert block.startswith(report.BEGIN_MARKER) and block.endswith(report.END_MARKER)
    doc = tmp_path / "validation-report.md"
    doc.write_text(f"# narrative\n\n{report.BEGIN_MARKER}\nold\n{report.END_MARKER}\n\ntail\n")
    assert report.main(["--quick", "--update", str(doc), "--json", str(tmp_path / "r.json")]) == 0
    text = doc.read_text()
    assert text.startswith("# narrative") and text.rstrip().endswith("tail") and "old" not in text
    assert os.path.getsize(tmp_path / "r.json") > 0
