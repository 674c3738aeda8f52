"""GPU checks of the tensor-core network kernels and the learned LSM regression.

Bars:
  * tcgen05 GEMM (BF16 in, FP32 accumulate) equals the BF16-rounded product to FP32
    summation accuracy.
  * One forward/backward pass: every gradient block within 2 % (relative L2) of
    the oracle evaluated with the same BF16 rounding points (the remainder is
    tanh.approx and FP32 summation order); inference within 1 % of the oracle.
  * Learned LSM: within 3 SE (+ the 50-date Bermudan gap allowance 0.02) of the
    CRR American tree, and its frozen policy replayed out of sample agrees with
    the in-sample price within 3 SE.
  * Gain over the method without it (the Laguerre QR regression): both exercise
    policies are learned on the same paths from S0 = 40 and replayed on common
    held-out paths (three fresh seeds) from several spots.  A better policy is
    worth more on the same paths, so the paired difference learned - QR is the
    gain.  In distribution it must not be negative beyond its noise; from deep
    in-the-money spots, where the cubic Laguerre fit extrapolates and keeps
    paths alive that should be exercised, the learned policy must recover the
    exercise value (tree price) and beat QR by a wide margin.
  * Batches: every contract of an uneven batch prices as it does alone.
"""
from __future__ import annotations

import numpy as np
import pytest

import mcd_gpu as G
import mlp_oracle as M

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30))


def test_umma_gemm_matches_bf16_product(engine):
    rng = np.random.default_rng(11)
    a = rng.standard_normal((128, 64)).astype(np.float32)
    b = rng.standard_normal((64, 64)).astype(np.float32)
    d = engine.umma_selftest(a, b)
    ref = M.bf16(a) @ M.bf16(b).T
    assert np.abs(d - ref).max() <= 1e-4 * np.abs(ref).max(), np.abs(d - ref).max()


@pytest.mark.parametrize("n", [128, 77])
def test_gradients_match_oracle(engine, n):
    rng = np.random.default_rng(n)
    p = M.init_params(rng)
    p[M.B1:M.W2] = rng.standard_normal(64) * 0.1
    p[M.B2:M.W3] = rng.standard_normal(64) * 0.1
    p = p.astype(np.float32).astype(np.float64)
    x0 = rng.uniform(-2, 0.5, n).astype(np.float32)
    x1 = rng.uniform(0, 1, n).astype(np.float32)
    y = rng.uniform(0, 0.3, n).astype(np.float32)
    w = (rng.uniform(size=n) > 0.3).astype(np.float32)
    g, loss = engine.mlp_gradients(p, x0, x1, y, w)
    ref_loss, ref = M.loss_and_grad(p, x0, x1, y, w, bf16_tc=True)
    assert abs(loss - ref_loss) <= 1e-2 * ref_loss
    for name, lo, hi in [("W1", M.W1, M.B1), ("b1", M.B1, M.W2), ("W2", M.W2, M.B2), ("b2", M.B2, M.W3),
                         ("W3", M.W3, M.B3), ("b3", M.B3, M.B3 + 1)]:
        err = rel_l2(g[lo:hi], ref[lo:hi])
        assert err <= 2e-2, (name, err)


def test_forward_matches_oracle(engine):
    rng = np.random.default_rng(5)
    p = M.init_params(rng).astype(np.float32)
    n = 1000
    x0 = rng.uniform(-2, 0.5, n).astype(np.float32)
    x1 = rng.uniform(0, 1, n).astype(np.float32)
    out = engine.mlp_forward(p, x0, x1)
    ref = M.forward(p.astype(np.float64), x0, x1, bf16_tc=True)
    assert rel_l2(out, ref) <= 1e-2


CASES = [(36, 40, .06, 0, .2, 1.0, 1), (40, 40, .06, 0, .4, 2.0, 1)]


@pytest.mark.parametrize("case", CASES)
def test_learned_lsm_against_tree_and_out_of_sample(engine, orc, case):
    s, k, r, q, v, t, ty = case
    paths, n = 1 << 17, 50
    res = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, 42, precision="fp32",
                                          regression="mlp")
    assert res.reserved == 0  # no QR fallback was needed
    tree = orc.orc_crr_binomial_american(s, k, r, q, v, t, 2000, ty)
    assert abs(res.price - tree) < 3 * res.standard_error + 0.02, (res.price, res.standard_error, tree)
    w, has = engine.mlp_policy(0, n)
    assert has[1:n].all()
    oos = engine.reprice_mlp(s, k, r, q, v, t, ty, n, paths, 4242, w, has, "fp32")
    assert abs(oos.price - res.price) < 3 * np.hypot(oos.standard_error, res.standard_error) + 0.01


def test_learned_policy_gains_over_qr_out_of_sample(engine, orc):
    s, k, r, q, v, t, ty = 40, 40, .06, 0, .2, 1.0, 1
    paths, n = 1 << 17, 50
    res = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, 42, precision="fp32", regression="mlp")
    assert res.reserved == 0
    w, has = engine.mlp_policy(0, n)
    qr, co, hq = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, 42, precision="fp32",
                                                 policy=True)
    seeds = (777, 778, 779)
    for s2 in (30, 32, 40, 44):
        mlp = np.array([engine.reprice_mlp(s2, k, r, q, v, t, ty, n, paths, sd, w, has, "fp32").price for sd in seeds])
        qro = np.array([engine.reprice_against_frozen_policy(s2, k, r, q, v, t, ty, n, paths, sd, co, hq, False,
                                                             "fp32") for sd in seeds])
        gain = mlp - qro
        tree = orc.orc_crr_binomial_american(s2, k, r, q, v, t, 2000, ty)
        print(f"S0={s2}: learned {mlp.mean():.5f}  QR {qro.mean():.5f}  gain {gain.mean():+.5f}  tree {tree:.5f}")
        if s2 <= 32:  # deep in the money: exercise at once is optimal
            assert abs(mlp.mean() - tree) < 0.01, (s2, mlp, tree)
            assert gain.mean() > 0.1, (s2, gain)
        else:
            assert gain.mean() > -0.002, (s2, gain)


def test_learned_training_runs_and_features_move(engine):
    # The network is trained on the GPU (Adam, tensor-core forward/backward):
    # the first-date snapshot's hidden layer differs from the seeded initial
    # weights after training, and is identical to them without training.
    s, k, r, q, v, t, ty = 36, 40, .06, 0, .2, 1.0, 1
    paths, n = 1 << 15, 10
    snaps = {}
    try:
        for steps in (0, 200):
            engine.set_mlp_config(steps, 0, 3e-3, 1e-3)
            res = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, 42, precision="fp32",
                                                  regression="mlp")
            assert res.reserved == 0
            w, has = engine.mlp_policy(0, n)
            snaps[steps] = w[n - 1].copy()
    finally:
        engine.set_mlp_config()
    moved = rel_l2(snaps[200][M.W2:M.B2], snaps[0][M.W2:M.B2])
    assert 1e-3 < moved < 1.0, moved


def test_learned_batch_matches_single(engine):
    cs = [(36, 40, .06, 0, .2, 1.0, 1, 10, 20000, 5), (44, 40, .06, 0, .4, 2.0, 1, 37, 70000, 6),
          (40, 40, .06, 0, .3, 0.5, 0, 23, 9000, 7)]
    arr = np.array(cs, dtype=G.LSM_CONTRACT_DTYPE)
    batch = engine.lsm_batch(arr, precision="fp32", regression="mlp")
    for i, c in enumerate(cs):
        one = engine.monte_carlo_lsm_american(*c, precision="fp32", regression="mlp")
        assert batch[i]["price"] == one.price, (i, batch[i]["price"], one.price)
        assert batch[i]["reserved"] == one.reserved


@pytest.mark.parametrize("case", [(40, 40, .06, 0, .2, 1.0, 1), (36, 40, .06, 0, .4, 2.0, 1),
                                  (100, 100, .05, .08, .3, 1.0, 0)])
def test_node_tables_agree_with_the_network_path_by_path(engine, case):
    """The fit decides exercise from node tables (each date's network at 512
    values of ln(S/K), interpolated); replaying the fitted networks path by path
    (mcd_lsm_reprice_mlp) on the same paths changes only decisions of paths that
    are nearly indifferent between exercising and holding.  Their realised cash
    flows move the in-sample price by a fraction of a standard error (0.05-0.3
    SE here, not shrinking with finer tables: about what the in-sample price
    moves when the basis changes at all), never by a standard error."""
    s, k, r, q, v, t, ty = case
    paths, n = 1 << 17, 50
    res = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, 42, precision="fp32", regression="mlp")
    assert res.reserved == 0
    w, has = engine.mlp_policy(0, n)
    same = engine.reprice_mlp(s, k, r, q, v, t, ty, n, paths, 42, w, has, "fp32")
    print(case, res.price, same.price, (same.price - res.price) / res.standard_error)
    assert abs(same.price - res.price) < 0.5 * res.standard_error


def test_learned_path_count_limit(engine, gpu_lib):
    """Bin moments are exact 64-bit integers up to 2^23 paths per CTA, so the
    learned regression refuses more than 2^31 paths per contract (before any
    allocation)."""
    c = np.zeros(1, dtype=gpu_lib.LSM_CONTRACT_DTYPE)
    c[0] = (40.0, 40.0, 0.06, 0.0, 0.2, 1.0, 1, 1, (1 << 31) + 1024, 1)
    with pytest.raises(gpu_lib.McdError, match="2\\^31"):
        engine.lsm_batch(c, "fp32", "mlp")
    c[0] = (40.0, 40.0, 0.06, 0.0, 0.2, 1.0, 1, 5, 0, 1)  # no paths to train on
    with pytest.raises(gpu_lib.McdError, match=">= 1"):
        engine.lsm_batch(c, "fp32", "mlp")


def test_learned_fp64_paths_and_fine_tuning(engine, orc):
    """The learned regression on FP64 paths (the binned pass in FP64) and with
    per-date fine-tuning of the features (steps > 0: node tables rebuilt from
    the updated network every date) both price the put within noise of the
    FP32 default and of the CRR tree."""
    s, k, r, q, v, t, ty = 40, 40, .06, 0, .2, 1.0, 1
    paths, n = 1 << 17, 50
    base = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, 42, precision="fp32", regression="mlp")
    f64 = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, 42, precision="fp64", regression="mlp")
    try:
        engine.set_mlp_config(300, 20, 3e-3, 1e-3)
        tuned = engine.monte_carlo_lsm_american(s, k, r, q, v, t, ty, n, paths, 42, precision="fp32",
                                                regression="mlp")
    finally:
        engine.set_mlp_config()
    tree = orc.orc_crr_binomial_american(s, k, r, q, v, t, 2000, ty)
    for res in (f64, tuned):
        assert res.reserved == 0
        assert abs(res.price - base.price) < 1.0 * base.standard_error, (res.price, base.price)
        assert abs(res.price - tree) < 3 * res.standard_error + 0.02, (res.price, tree)


@pytest.mark.parametrize("n_dates, paths", [(1, 50000), (2, 50000), (5, 3), (3, 1)])
def test_learned_edge_cases(engine, n_dates, paths):
    """One exercise date (no regression: the terminal payoff discounted), two
    dates (one fit), and path counts too small for a fit (fewer than 4 paths
    in the money: no exercise at that date).  The learned regression prices
    these like the QR regression where no fit is involved, and never fails."""
    c = (38.0, 40.0, 0.06, 0.0, 0.25, 1.0, 1, n_dates, paths, 9)
    ml = engine.monte_carlo_lsm_american(*c, precision="fp32", regression="mlp")
    qr = engine.monte_carlo_lsm_american(*c, precision="fp32", regression="qr")
    assert np.isfinite(ml.price) and np.isfinite(ml.standard_error) and ml.reserved == 0
    if n_dates == 1 or paths < 4:
        assert abs(ml.price - qr.price) <= 1e-6 * max(1.0, abs(qr.price)), (ml.price, qr.price)
    else:
        assert abs(ml.price - qr.price) < 3 * qr.standard_error + 0.02, (ml.price, qr.price)
