"""The benchmark configurations checked at their stated sizes (FP32 paths).

* Heston QE: parameter sets drawn from the configuration's ranges (kappa
  U[0.5,3], theta U[0.02,0.09], xi U[0.2,1.0], rho U[-0.9,-0.3], v0
  U[0.01,0.09], S0 100, r 0.03, T 1), 64 strikes in [70,130], 252 steps, 2^20
  paths: every 16th of the 256 benchmark sets against the semi-analytic price
  (the reference's heston_semi_analytic, src/pricers/heston.cpp:48-82).
* Batched risk: the FP32 Greeks of a per-product sample of the 1024 benchmark
  contracts (Asian/barrier, 252 steps, 2^18 paths, CRN finite differences with
  1e-4 relative bumps, pathwise and likelihood-ratio Greeks) against the same
  launch in FP64 -- the reference's arithmetic on the same draws: within 0.1
  SE, finite-difference gamma within 1 SE.
"""
from __future__ import annotations

import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def heston_sets(M, n_sets=256):
    """The benchmark's parameter sets (numpy default_rng(42), in this order)."""
    rng = np.random.default_rng(42)
    sets = np.zeros(n_sets, dtype=M.HESTON_DTYPE)
    sets["spot"] = 100.0
    sets["rate"] = 0.03
    sets["kappa"] = rng.uniform(0.5, 3.0, n_sets)
    sets["theta"] = rng.uniform(0.02, 0.09, n_sets)
    sets["xi"] = rng.uniform(0.2, 1.0, n_sets)
    sets["rho"] = rng.uniform(-0.9, -0.3, n_sets)
    sets["v0"] = rng.uniform(0.01, 0.09, n_sets)
    sets["time"] = 1.0
    return sets


def test_heston_configuration_against_semi_analytic(engine, gpu_lib):
    M = gpu_lib
    sets = heston_sets(M)[::16]
    strikes = np.linspace(70.0, 130.0, 64)
    out = engine.heston_qe_batch(sets, strikes, 0, 252, 1 << 20, 42, "fp32")
    z = np.zeros((len(sets), len(strikes)))
    for i, s in enumerate(sets):
        hp = M.HestonParams(*[float(s[f]) for f in M.HESTON_DTYPE.names])
        for j, k in enumerate(strikes):
            exact = M.heston_semi_analytic(hp, float(k), 0)
            z[i, j] = (out["price"][i, j] - exact) / out["standard_error"][i, j]
    worst = np.unravel_index(np.abs(z).argmax(), z.shape)
    print(f"Heston QE vs semi-analytic over {z.size} prices: max |z| {np.abs(z).max():.2f} "
          f"(set {worst[0] * 16}, K {strikes[worst[1]]:.1f}), mean z {z.mean():+.3f}, "
          f"share |z| > 3: {(np.abs(z) > 3).mean():.4f}")
    # every price within 3 SE (the strikes of one set share their paths, so
    # their z-scores move together; the mean over 16 sets is not a test)
    assert np.abs(z).max() < 3.0


def test_risk_configuration_fp32_against_fp64(engine, gpu_lib):
    import bench
    c = bench.risk_batch()[::32]
    assert len(c) == 32 and (c["monitoring_points"] == 252).all() and (c["path_count"] == 1 << 18).all()
    r32 = engine.greeks_batch(c, 1e-4, 1e-4, "fp32")
    r64 = engine.greeks_batch(c, 1e-4, 1e-4, "fp64")
    worst = {}
    for name in gpu_lib.GREEK_NAMES:
        se = r64[name][:, 1]
        ok = se > 0
        if not ok.any():
            continue
        err = np.abs(r32[name][ok, 0] - r64[name][ok, 0]) / se[ok]
        worst[name] = float(err.max())
    print("FP32 vs FP64 Greeks, max error in FP64 standard errors:",
          {k: round(v, 4) for k, v in worst.items()})
    # Finite-difference gamma at a 1e-4 bump is carried by the few paths
    # whose barrier or strike test changes between the bumped spots (each adds
    # ~payoff / h^2); FP32 path rounding moves such a path across a boundary
    # now and then, which shifts the estimate by up to about one of its
    # standard errors.  Every other output stays within a tenth of one.
    for name, w in worst.items():
        assert w <= (1.0 if name == "fd_gamma" else 0.1), (name, w)
