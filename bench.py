#!/usr/bin/env python3
"""Benchmark: batched path-dependent GBM pricing on one GB300.

Workload (the reference's batched path-dependent configuration): 4096 GBM
contracts in one launch -- arithmetic/geometric x fixed/floating x call/put
Asians, all 8 barrier types, fixed/floating lookbacks and cash digitals --
with S0=100, K~U[80,120], sigma~U[.1,.5], r~U[0,.06], T~U[.25,2], monitoring
steps ~U{12..252}, paths log-uniform in [1e4, 1e6], seed 42+i.  Barrier levels
H = S0(1 +/- U[.05,.3]), rebate 0.  Parameters come from numpy's default_rng(42)
(synthetic data with the configuration's distributions).

A step prices the whole batch once: FP32 paths, FP64 accumulation, one
persistent-kernel launch (plus the fixed-order merge) replayed from a CUDA
graph.  `value` is paths/s with the batch resident on the device; `e2e` is the
same metric through the C ABI with host arrays (copies inside the timed
region).  The L2 is flushed (256 MB write) between timed steps.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "derivative-pricing_gb300")
sys.path.insert(0, PKG)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "paths_per_second"
UNIT = "paths/s"
WORKLOAD = "batch of 4096 path-dependent GBM contracts (asian/barrier/lookback/digital), FP32 paths"


def make_batch(n=4096, seed=42, rank=0):
    """The configuration's contract list (mcd_contract records).  Replica `rank`
    of a multi-GPU run prices the same contract terms on its own pricing seeds
    (42 + rank n + i), so N ranks price a book N times the size (weak scaling)."""
    import mcd_gpu as M
    rng = np.random.default_rng(seed)
    c = M.contracts(n)
    variants = []
    for avg in (0, 1):
        for style in (0, 1):
            for ty in (0, 1):
                variants.append(dict(product=M.ASIAN, average_style=avg, strike_style=style, type=ty))
    for d in (0, 1):
        for k in (0, 1):
            for ty in (0, 1):
                variants.append(dict(product=M.BARRIER, direction=d, knock=k, type=ty))
    for style in (0, 1):
        for ty in (0, 1):
            variants.append(dict(product=M.LOOKBACK, strike_style=style, type=ty))
    for ty in (0, 1):
        variants.append(dict(product=M.DIGITAL, digital_style=0, type=ty))
    pick = rng.integers(0, len(variants), n)
    for i, v in enumerate(pick):
        for k, val in variants[v].items():
            c[k][i] = val
    c["spot"] = 100.0
    c["strike"] = rng.uniform(80, 120, n)
    c["vol"] = rng.uniform(0.1, 0.5, n)
    c["rate"] = rng.uniform(0.0, 0.06, n)
    c["time"] = rng.uniform(0.25, 2.0, n)
    c["monitoring_points"] = rng.integers(12, 253, n)
    c["path_count"] = np.round(10.0 ** rng.uniform(4, 6, n)).astype(np.uint64)
    h = rng.uniform(0.05, 0.3, n)
    c["barrier"] = np.where(c["direction"] == 0, 100.0 * (1 + h), 100.0 * (1 - h))
    c["rebate"] = 0.0
    c["cash_amount"] = 1.0
    c["seed"] = 42 + np.uint64(rank * n) + np.arange(n, dtype=np.uint64)
    return c


def max_over_ranks(x, device="cpu"):
    """The largest of every rank's x (the job's time is its slowest rank's)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def path_steps(c):
    steps = np.where(c["product"] == 1, 1, c["monitoring_points"]).astype(np.float64)
    return float((steps * c["path_count"].astype(np.float64)).sum())


# The path kernel's instruction count and DRAM traffic, measured by ncu on the
# 256-contract case (`bench.py --case path --launch-shape V,0`: the second
# price_batch launch, metrics smsp__inst_executed.sum, dram__bytes_read.sum and
# dram__bytes_write.sum) for each register variant V, together with the digest
# of the sources they were measured on.  The roofline below uses them only
# while the sources still have that digest; otherwise it reports the
# instruction-based figures as unmeasured (null) rather than stale.
PATH_KERNEL_SOURCES = ("derivative-pricing_gb300/csrc/gbm_paths.cu",
                       "derivative-pricing_gb300/csrc/device_common.cuh",
                       "derivative-pricing_gb300/csrc/engine.hpp")
PATH_KERNEL_PROFILE = {
    "sources": "bd4a0512aa792e85",
    "case_path_steps": 6807363601.0,
    # variant -> smsp__inst_executed.sum of one launch
    "warp_inst": {"0": 15205895145, "1": 16932465571, "2": 19960539871, "3": 15461878018, "4": 15332180663},
    # variant -> dram__bytes_read.sum + dram__bytes_write.sum of one launch
    "dram_bytes": {"0": 514560, "1": 525312, "2": 698880, "3": 3397120, "4": 473856},
}


def sources_digest(paths=PATH_KERNEL_SOURCES):
    import hashlib
    h = hashlib.sha256()
    for rel in paths:
        with open(os.path.join(ROOT, rel), "rb") as f:
            h.update(f.read())
    return h.hexdigest()[:16]


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled while the timed region runs."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.device = device
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.QUERY,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) >= 9:
                self.rows.append(parts)

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        sm = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


def cpu_baseline_sample(c, budget_s=12.0):
    """Times the CPU port (bit-identical restatement of the reference) on a
    stratified sample of the batch, each contract on all host threads over the
    reference's fixed chunk partition (its own multithreaded path).  The rate
    is measured in path-steps/s, which does not depend on the sample's mix of
    step counts, and turned into the full batch's paths/s through the batch's
    own path-steps per path (the time the CPU would take for the whole batch)."""
    import oracle as O
    orc = O.load()
    threads = os.cpu_count() or 1
    order = np.argsort(c["monitoring_points"] * c["path_count"].astype(np.float64))
    # Grow a stratified sample (every k-th contract by cost) until ~budget_s of work.
    for k in (512, 256, 128, 64):
        idx = order[::k]
        est = path_steps(c[idx]) / (threads * 1.2e7)
        if est >= budget_s / 2 or k == 64:
            break
    sample = c[idx]
    arr = (O.Contract * len(sample))()
    for i, row in enumerate(sample):
        for name in row.dtype.names:
            setattr(arr[i], name, row[name].item())
    out = (O.McResult * len(sample))()
    t0 = time.perf_counter()
    orc.orc_price_batch(arr, len(sample), threads, 0, out)
    dt = time.perf_counter() - t0
    paths = float(sample["path_count"].astype(np.float64).sum())
    rate = path_steps(sample) / dt
    full_s = path_steps(c) / rate
    return {"value": float(c["path_count"].astype(np.float64).sum()) / full_s, "unit": UNIT, "cores": threads,
            "kind": "port",
            "sample": f"{len(sample)} of {len(c)} contracts (every {k}th by cost), {paths:.3g} paths, "
                      f"{path_steps(sample):.3g} path-steps, {dt:.2f} s; paths/s of the whole batch at the "
                      f"sample's path-steps/s",
            "path_steps_per_s": rate, "full_batch_s_extrapolated": full_s,
            "build": "oracle/Makefile: -O3, -mcpu=native on aarch64 (-march=native elsewhere), "
                     "-ffp-contract=off"}


def lsm_grid():
    """The American-put grid: S0 in {36,38,40,42,44}, K=40, r=.06, sigma in {.2,.4},
    T in {1,2}, 50 exercise dates, 2^20 paths, seed 42+i."""
    import mcd_gpu as M
    rows = [(s, 40.0, 0.06, 0.0, v, t, 1, 50, 1 << 20, 42 + i)
            for i, (s, v, t) in enumerate((s, v, t) for s in (36, 38, 40, 42, 44) for v in (0.2, 0.4) for t in (1.0, 2.0))]
    return np.array(rows, dtype=M.LSM_CONTRACT_DTYPE)


def _timed(fn, reps=2):
    fn()
    ts = []
    out = None
    for _ in range(reps):
        t0 = time.perf_counter()
        out = fn()
        ts.append(time.perf_counter() - t0)
    return out, min(ts)


def lsm_algorithmic_bytes(g):
    """Algorithmic HBM bytes of Longstaff-Schwartz per contract: N (4 (D+1) +
    20 D) -- the FP32 paths written once, one date column read and FP64 cash
    flows read and written per date."""
    n = g["path_count"].astype(np.float64)
    d = g["monitoring_points"].astype(np.float64)
    return float((n * (4.0 * (d + 1) + 20.0 * d)).sum())


def hbm_roofline(bytes_, seconds, peaks):
    peak = peaks.get("hbm_gbs")
    achieved = bytes_ / seconds / 1e9
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if peak else None, "algorithmic_bytes": bytes_,
            "peak_source": "MEASURED_PEAKS.json hbm_gbs (measured)" if peak else None,
            "note": "algorithmic bytes over the wall time of the whole call (forward simulation, "
                    "backward pass, copies)"}


def bench_lsm(eng, peaks):
    """Time-to-price of the 20-put grid: plain FP64 GPU path (QR, FP64 paths),
    FP32 QR, and the learned regression (FP32 paths, BF16 tensor-core network).
    Errors are measured against the FP64 result (the reference's arithmetic,
    parity-tested to 1e-12 at this size) in units of its standard error, and
    against the exact 50-date Bermudan value (a 5000-step CRR lattice with
    exercise at the LSM dates)."""
    g = lsm_grid()
    r64, t64 = _timed(lambda: eng.lsm_batch(g, "fp64", "qr"))
    r32, t32 = _timed(lambda: eng.lsm_batch(g, "fp32", "qr"))
    rml, tml = _timed(lambda: eng.lsm_batch(g, "fp32", "mlp"))
    t0 = time.perf_counter()
    rml64 = eng.lsm_batch(g, "fp64", "mlp")  # the learned method's own FP64 arithmetic (FP64 paths)
    tml64 = time.perf_counter() - t0
    import mcd_gpu as M
    se = r64["standard_error"]
    e32 = np.abs(r32["price"] - r64["price"]) / se
    eml = np.abs(rml["price"] - r64["price"]) / se
    eml64 = np.abs(rml["price"] - rml64["price"]) / rml64["standard_error"]
    tree = np.array([M.crr_binomial_american(r["spot"], r["strike"], r["rate"], r["carry_yield"], r["vol"],
                                             r["time"], 2000, 1) for r in g])
    berm = np.array([M.crr_binomial_bermudan(r["spot"], r["strike"], r["rate"], r["carry_yield"], r["vol"],
                                             r["time"], int(r["monitoring_points"]), 100, 1) for r in g])
    # Out of sample: both fitted policies replayed on the same fresh paths
    # (seed + 10^7), so foresight bias is gone and the better policy earns more.
    mlp_pol = [eng.mlp_policy(i, int(r["monitoring_points"])) for i, r in enumerate(g)]
    oos_qr, oos_ml, oos_se = [], [], []
    for r, (w, has) in zip(g, mlp_pol):
        args = (r["spot"], r["strike"], r["rate"], r["carry_yield"], r["vol"], r["time"], int(r["type"]),
                int(r["monitoring_points"]))
        _, co, hq = eng.monte_carlo_lsm_american(*args, int(r["path_count"]), int(r["seed"]), precision="fp64",
                                                 policy=True)
        fresh = int(r["seed"]) + 10_000_000
        oos_qr.append(eng.reprice_against_frozen_policy(*args, int(r["path_count"]), fresh, co, hq, False, "fp64"))
        ml_oos = eng.reprice_mlp(*args, int(r["path_count"]), fresh, w, has, "fp32")
        oos_ml.append(ml_oos.price)
        oos_se.append(ml_oos.standard_error)
    gain = (np.array(oos_ml) - np.array(oos_qr)) / np.array(oos_se)
    zb = lambda p: (p - berm) / se  # noqa: E731
    nbytes = lsm_algorithmic_bytes(g)
    return {"workload": "20 American puts (S0 36..44, sigma .2/.4, T 1/2), 50 dates, 2^20 paths each",
            "fp64_qr_s": t64, "fp32_qr_s": t32, "learned_s": tml,
            "speedup_learned_over_fp64": t64 / tml, "speedup_fp32_qr_over_fp64": t64 / t32,
            "learned_err_vs_fp64_max_se": float(eml.max()), "learned_err_vs_fp64_mean_se": float(eml.mean()),
            "learned_minus_fp64_mean_se": float(((rml["price"] - r64["price"]) / se).mean()),
            "fp32_qr_err_vs_fp64_max_se": float(e32.max()),
            "learned_vs_learned_fp64": {
                "note": "the learned regression on FP32 paths against the same method on FP64 paths (its own "
                        "FP64 oracle: FP64 paths, exercise tests and cash flows), |difference| / SE; the "
                        "errors above compare against the QR regression's price, a different policy",
                "max_se": float(eml64.max()), "mean_se": float(eml64.mean()), "fp64_learned_s": tml64},
            "learned_fallbacks": int((rml["reserved"] != 0).sum()),
            "roofline_fp32_qr": hbm_roofline(nbytes, t32, peaks),
            "roofline_learned": hbm_roofline(nbytes, tml, peaks),
            "vs_bermudan_lattice": {
                "note": "z = (in-sample LSM price - exact 50-date Bermudan value) / SE; the lattice is the "
                        "value LSM estimates, so |z| follows the Monte Carlo error plus each regression's "
                        "policy loss and foresight bias",
                "fp64_qr_max_abs_z": float(np.abs(zb(r64["price"])).max()),
                "fp64_qr_mean_abs_z": float(np.abs(zb(r64["price"])).mean()),
                "fp32_qr_max_abs_z": float(np.abs(zb(r32["price"])).max()),
                "learned_max_abs_z": float(np.abs(zb(rml["price"])).max()),
                "learned_mean_abs_z": float(np.abs(zb(rml["price"])).mean()),
                "learned_mean_z": float(zb(rml["price"]).mean()), "fp64_qr_mean_z": float(zb(r64["price"]).mean())},
            "vs_crr_tree_2000": {
                "note": "in-sample LSM prices against the American lattice price; the 50-date Bermudan "
                        "and the in-sample foresight bias both enter",
                "fp64_qr_mean_abs_err": float(np.mean(np.abs(r64["price"] - tree))),
                "fp32_qr_mean_abs_err": float(np.mean(np.abs(r32["price"] - tree))),
                "learned_mean_abs_err": float(np.mean(np.abs(rml["price"] - tree))),
                "mean_se": float(np.mean(se))},
            "out_of_sample": {
                "note": "the learned policy (FP32 replay) and the FP64 QR policy (FP64 replay) on the same "
                        "fresh 2^20 paths per put; difference learned - QR in units of the replay's standard error",
                "learned_minus_qr_min_se": float(gain.min()), "learned_minus_qr_mean_se": float(gain.mean()),
                "learned_minus_qr_max_se": float(gain.max()),
                "learned_mean_abs_err_vs_bermudan": float(np.mean(np.abs(np.array(oos_ml) - berm))),
                "qr_mean_abs_err_vs_bermudan": float(np.mean(np.abs(np.array(oos_qr) - berm)))},
            "timing": "wall clock of one mcd_lsm_batch call (host arrays, graph capture and copies included), "
                      "best of 2 after a warm-up"}


def risk_batch(n=1024, seed=42):
    """Asian/barrier contracts drawn as in the batch configuration, 252 steps, 2^18 paths."""
    c = make_batch(4 * n, seed)
    c = c[np.isin(c["product"], [2, 3])][:n].copy()
    c["monitoring_points"] = 252
    c["path_count"] = 1 << 18
    return c


def bench_risk(eng, peaks):
    """Batched risk: price, CRN finite-difference delta/gamma/vega (bump 1e-4
    relative), pathwise and likelihood-ratio Greeks of 1024 Asian/barrier
    contracts in one graph launch; learned LSM on 512 American puts with
    uneven date counts U{10..100}, 2^18 paths, and their frozen-boundary
    delta/gamma/vega."""
    import mcd_gpu as M
    c = risk_batch()
    v, ctas, _ = eng.greeks_autotune(c, 1e-4, 1e-4, "fp32")  # on the batch itself, as the path engine
    res, tg = _timed(lambda: eng.greeks_batch(c, 1e-4, 1e-4, "fp32"))
    steps = float(len(c)) * 252 * (1 << 18)
    rng = np.random.default_rng(7)
    n = 512
    puts = np.zeros(n, dtype=M.LSM_CONTRACT_DTYPE)
    puts["spot"] = rng.uniform(36, 44, n)
    puts["strike"] = 40.0
    puts["rate"] = 0.06
    puts["vol"] = rng.uniform(0.2, 0.4, n)
    puts["time"] = rng.uniform(0.5, 2.0, n)
    puts["type"] = 1
    puts["monitoring_points"] = rng.integers(10, 101, n)
    puts["path_count"] = 1 << 18
    puts["seed"] = 1000 + np.arange(n)
    ml, tl = _timed(lambda: eng.lsm_batch(puts, "fp32", "mlp"), reps=1)
    qr, tq = _timed(lambda: eng.lsm_batch(puts, "fp32", "qr"), reps=1)
    ag, ta = _timed(lambda: eng.lsm_greeks_batch(puts, 0.01, 0.01, "fp32"), reps=1)
    # FP32 against FP64 (the reference's arithmetic, same draws) on every 32nd contract
    sub = c[::32]
    g32 = eng.greeks_batch(sub, 1e-4, 1e-4, "fp32")
    g64 = eng.greeks_batch(sub, 1e-4, 1e-4, "fp64")
    fp32_err = {}
    for name in M.GREEK_NAMES:
        ok = g64[name][:, 1] > 0
        if ok.any():
            fp32_err[name] = float((np.abs(g32[name][ok, 0] - g64[name][ok, 0]) / g64[name][ok, 1]).max())
    return {"greeks": {"contracts": len(c), "s": tg, "contracts_per_second": len(c) / tg,
                       "path_steps_per_second": steps / tg, "launch_shape": {"variant": v, "ctas_per_sm": ctas},
                       "outputs": "price, FD delta/gamma/vega, pathwise delta/vega/rho, LR delta/gamma/vega/rho",
                       "fp32_err_vs_fp64_max_se": fp32_err,
                       "fp32_err_sample": f"{len(sub)} contracts (every 32nd), same launch in FP64"},
            "learned_lsm_512": {"s": tl, "contracts_per_second": n / tl, "qr_s": tq,
                                "roofline": hbm_roofline(lsm_algorithmic_bytes(puts), tl, peaks),
                                "roofline_qr": hbm_roofline(lsm_algorithmic_bytes(puts), tq, peaks),
                                "max_abs_diff_vs_qr_in_se": float(np.max(np.abs(ml["price"] - qr["price"]) /
                                                                         qr["standard_error"])),
                                "fallbacks": int((ml["reserved"] != 0).sum())},
            "american_greeks_512": {"s": ta, "contracts_per_second": n / ta,
                                    "outputs": "QR fit, then price/delta/gamma/vega against the frozen policy "
                                               "(bumps 1% of spot and vol), all scenarios in one streaming pass",
                                    "mean_delta_se": float(np.mean(ag["delta"][:, 1]))}}


def bench_heston(eng, n_sets=256):
    """Heston QE: parameter sets drawn from the configuration's ranges, 64
    strikes linspace(70,130) each, 252 steps, 2^20 paths, FP32 paths."""
    import mcd_gpu as M
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
    strikes = np.linspace(70.0, 130.0, 64)
    out, t = _timed(lambda: eng.heston_qe_batch(sets, strikes, 0, 252, 1 << 20, 42, "fp32"), reps=1)
    steps = float(n_sets) * 252 * (1 << 20)
    # every price against the semi-analytic Heston price (the configuration's check)
    z = np.zeros((n_sets, len(strikes)))
    for i, row in enumerate(sets):
        hp = M.HestonParams(*[float(row[f]) for f in M.HESTON_DTYPE.names])
        for j, k in enumerate(strikes):
            z[i, j] = (out["price"][i, j] - M.heston_semi_analytic(hp, float(k), 0)) / out["standard_error"][i, j]
    return {"sets": n_sets, "strikes": 64, "s": t, "paths_per_second": n_sets * (1 << 20) / t,
            "path_steps_per_second": steps / t, "prices_per_second": n_sets * 64 / t,
            "vs_semi_analytic": {"prices": int(z.size), "max_abs_z": float(np.abs(z).max()),
                                 "mean_z": float(z.mean()), "share_abs_z_over_3": float((np.abs(z) > 3).mean()),
                                 "note": "z = (QE price - semi-analytic price) / SE, FP32 paths, 252 steps"}}


def bench_qmc(eng, c):
    """The Sobol + Brownian-bridge variant of the batch (dims = steps)."""
    q = c.copy()
    q["antithetic"] = 0
    q["control_variate"] = 0
    q["brownian_bridge"] = 0
    _, t = _timed(lambda: eng.qmc_batch(q, "fp32"))
    return {"s": t, "paths_per_second": float(q["path_count"].astype(np.float64).sum()) / t,
            "path_steps_per_second": path_steps(q) / t,
            "timing": "wall clock of one mcd_qmc_batch call (host arrays), best of 2 after a warm-up"}


def bench_european_1e6(eng):
    """The reference's CPU-runnable case: European call S0 = K = 100, r = 0.05,
    q = 0, sigma = 0.2, T = 1, 1e6 paths, seed 42, the reference's FP64
    arithmetic (its own output: price 10.463094885721839, SE 0.014739648351400047)
    and the FP32 path beside it; one pricer call each, host arguments, wall clock."""
    args = (100.0, 100.0, 0.05, 0.0, 0.2, 1.0, 0, 10**6, 42)
    out = {}
    for prec in ("fp64", "fp32"):
        r, t = _timed(lambda: eng.monte_carlo_european(*args, precision=prec), reps=5)
        out[prec] = {"s": t, "paths_per_second": 1e6 / t, "price": r.price, "standard_error": r.standard_error}
    out["reference_price"] = 10.463094885721839
    out["black_scholes"] = 10.450583572185565
    out["fp64_rel_diff_vs_reference"] = abs(out["fp64"]["price"] - 10.463094885721839) / 10.463094885721839
    return out


PROFILE_CASES = ("path", "greeks", "qmc", "heston", "lsm", "lsm_grid", "mlp", "mlp_grid", "american_greeks")


def run_case(case, launch_shape=None):
    """Small fixed workloads for profiling one kernel family (each priced twice:
    the second launch is the one to capture).  Sizes keep an ncu capture short:
      path      256 contracts of the batch configuration (FP32)
      greeks    64 Asian/barrier contracts, 252 steps, 2^16 paths (FP32)
      qmc       256 contracts of the batch configuration under Sobol + bridge
      heston    32 parameter sets x 64 strikes, 252 steps, 2^18 paths (8192 items: fills the GPU)
      lsm       4 puts of the American grid (2^20 paths, 50 dates), FP32 QR
      lsm_grid  the 20-put grid, FP32 QR
      mlp       4 puts of the grid, learned regression
      mlp_grid  the 20-put grid, learned regression
      american_greeks  the 20-put grid: QR fit, then frozen-boundary Greeks (FP32)"""
    import mcd_gpu as M
    eng = M.Engine(0)
    if launch_shape:
        v, cps = (int(x) for x in launch_shape.split(","))
        eng.set_launch_shape("fp32", v, cps)
    for _ in range(2):
        if case == "path":
            r = eng.price_batch(make_batch(256), "fp32")["price"]
        elif case == "greeks":
            c = risk_batch(64)
            c["path_count"] = 1 << 16
            r = eng.greeks_batch(c, 1e-4, 1e-4, "fp32")["fd_delta"][:, 0]
        elif case == "qmc":
            r = eng.qmc_batch(make_batch(256), "fp32")["price"]
        elif case == "heston":
            rng = np.random.default_rng(1)
            n = 32
            sets = np.zeros(n, dtype=M.HESTON_DTYPE)
            sets["spot"], sets["rate"], sets["time"] = 100.0, 0.03, 1.0
            sets["kappa"] = rng.uniform(0.5, 3.0, n)
            sets["theta"] = rng.uniform(0.02, 0.09, n)
            sets["xi"] = rng.uniform(0.2, 1.0, n)
            sets["rho"] = rng.uniform(-0.9, -0.3, n)
            sets["v0"] = rng.uniform(0.01, 0.09, n)
            r = eng.heston_qe_batch(sets, np.linspace(70.0, 130.0, 64), 0, 252, 1 << 18, 42, "fp32")["price"][0]
        elif case in ("lsm", "lsm_grid", "mlp", "mlp_grid"):
            g = lsm_grid()
            if case in ("lsm", "mlp"):
                g = g[:4]
            r = eng.lsm_batch(g, "fp32", "mlp" if case.startswith("mlp") else "qr")["price"]
        elif case == "american_greeks":
            r = eng.lsm_greeks_batch(lsm_grid(), 0.01, 0.01, "fp32")["delta"][:, 0]
        else:
            raise SystemExit(f"unknown case {case!r}; one of {PROFILE_CASES}")
    print(case, np.asarray(r)[:4])
    eng.close()
    return 0


def run_reference(args):
    """--impl reference: the reference's CPU algorithm (the oracle port,
    bit-identical to the reference built from source) on the host cores."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    c = make_batch()
    for _ in range(max(args.warmup, 0)):
        cpu_baseline_sample(c, budget_s=4.0)
    vals = []
    last = None
    for _ in range(max(args.steps, 1)):
        last = cpu_baseline_sample(c, budget_s=4.0)
        vals.append(last["value"])
    value = statistics.mean(vals)
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": WORKLOAD, "sample": last["sample"]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": last["cores"], "kind": "port",
                             "sample": last["sample"]},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--no-fp64", action="store_true", help="skip the FP64 comparison leg")
    ap.add_argument("--no-tune", action="store_true", help="keep the default launch shape")
    ap.add_argument("--launch-shape", metavar="VARIANT,CTAS_PER_SM",
                    help="use this launch shape of the path kernel instead of autotuning")
    ap.add_argument("--case", choices=PROFILE_CASES,
                    help="run one small profiling workload (see run_case) instead of the benchmark")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the LSM, risk, Heston and QMC sections")
    ap.add_argument("--contracts", type=int, default=4096,
                    help="batch size (the configuration is 4096; smaller only for profiling)")
    args = ap.parse_args()
    if args.case:
        return run_case(args.case, args.launch_shape)
    if args.impl == "reference":
        return run_reference(args)

    import torch
    import mcd_gpu as M

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    # Replicas: every rank prices its own batch (same terms, its own seeds); the
    # path has no exchange step, so no collective touches the data.
    c = make_batch(args.contracts, rank=rank)
    n = len(c)
    total_paths = float(c["path_count"].astype(np.float64).sum())
    total_steps = path_steps(c)

    eng = M.Engine(local)
    # Autotune the launch shape on the batch itself: on cost-stratified subsets
    # (a quarter, a sixteenth) the tail of the persistent launch ranked shapes
    # within 2 % of one another differently from the full batch.
    tune = c
    if args.launch_shape:
        v, cps = (int(x) for x in args.launch_shape.split(","))
        eng.set_launch_shape("fp32", v, cps)
        variant, ctas = eng.launch_shape("fp32")
    elif args.no_tune:
        variant, ctas = eng.launch_shape("fp32")
    else:
        variant, ctas, _ = eng.autotune(tune, "fp32")

    d_contracts = torch.from_numpy(c.view(np.uint8).copy()).cuda()
    d_results = torch.zeros(n * M.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device="cuda")
    # A dedicated stream: the library launches on it and the events below
    # are recorded on it (the legacy default stream has handle 0, which the
    # C ABI reads as "the context's own stream").
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)

    def step():
        eng.price_batch_device(d_contracts.data_ptr(), n, d_results.data_ptr(), "fp32",
                               stream.cuda_stream)

    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    eng.kernel_timing(reset=True)
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    with ClockSampler(local) as clocks:
        for i in range(args.steps):
            flush.zero_()
            starts[i].record(stream)
            step()
            ends[i].record(stream)
        torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = sum(step_ms) / len(step_ms)
    ms = max_over_ranks(ms, device="cuda")
    kernel_ms, launches = eng.kernel_timing(reset=True)
    if not kernel_ms > 0:
        raise RuntimeError("no kernel timing was collected")
    results = np.frombuffer(d_results.cpu().numpy().tobytes(), dtype=M.RESULT_DTYPE)
    assert (results["path_count"] == c["path_count"]).all()

    # End to end through the C ABI: host contracts in, host results out.
    host_out = np.zeros(n, dtype=M.RESULT_DTYPE)
    e2e_ms = []
    for i in range(args.warmup + args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        host_out = eng.price_batch(c, "fp32")
        t1 = time.perf_counter()
        if i >= args.warmup:
            e2e_ms.append((t1 - t0) * 1e3)
    e2e = max_over_ranks(sum(e2e_ms) / len(e2e_ms), device="cuda")
    assert host_out.tobytes() == results.tobytes(), "device-resident and host paths disagree"

    line = {
        "metric": METRIC, "value": world * total_paths / (ms / 1e3), "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32 paths / f64 accumulation",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "contracts": n, "total_paths": total_paths,
                   "total_path_steps": total_steps, "parallelism": f"replicas x{world}",
                   "l2": "flushed (256 MB write) between timed steps",
                   "launch_shape": {"variant": variant, "ctas_per_sm": ctas}},
        "contracts_per_second": world * n / (ms / 1e3),
        "path_steps_per_second": world * total_steps / (ms / 1e3),
        # per step: the contract digest, the persistent path kernel and the merge
        "gpu_launches": 3 * args.steps,
        "e2e": {"value": world * total_paths / (e2e / 1e3), "unit": UNIT,
                "h2d_bytes_per_step": n * 152 + (n + 1) * 4,
                "d2h_bytes_per_step": n * M.RESULT_DTYPE.itemsize + 8},
    }
    # Roofline of the persistent path kernel.  It is ALU-bound (no path data in
    # memory), so the bound is instruction issue: 4 SMSPs x 1 warp-instruction
    # per clock per SM at the SM clock sampled during the timed region.  The
    # instructions per path-step and the DRAM bytes per contract come from the
    # ncu capture of the same sources and register variant (PATH_KERNEL_PROFILE).
    peaks = {}
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            peaks = json.load(f)
    except OSError:
        pass
    sm_count = torch.cuda.get_device_properties(local).multi_processor_count
    clk = clocks.summary()
    mhz = clk["sm_mhz"] or peaks.get("sm_max_mhz", 2070.0)
    peak = sm_count * 4 * mhz * 1e6 / 1e12
    prof = PATH_KERNEL_PROFILE
    digest = sources_digest()
    fresh = prof["sources"] == digest and str(variant) in prof["warp_inst"]
    inst_per_step = (prof["warp_inst"][str(variant)] * 32.0 / prof["case_path_steps"]) if fresh else None
    achieved = (total_steps * inst_per_step / 32.0 / (kernel_ms / 1e3) / 1e12) if fresh else None
    line["roofline"] = {
        "bound": "alu", "achieved": achieved, "peak": peak, "unit": "Twarp-inst/s",
        "frac": (achieved / peak) if fresh else None,
        "traffic": (prof["dram_bytes"][str(variant)] * n / 256.0) if fresh else None,
        "kernel_ms": kernel_ms, "launches": launches,
        "path_steps_per_second_kernel": total_steps / (kernel_ms / 1e3),
        "inst_per_path_step": inst_per_step, "sources_digest": digest, "profiled_digest": prof["sources"],
        "note": "issue-slot roofline (4 warp-inst/clk/SM at the sampled SM clock); thread-instructions per "
                "path-step and DRAM bytes from an ncu capture of these sources and this register variant "
                "(256 contracts, traffic scaled by contracts); null when the sources changed since; "
                "no HBM or tensor-core bound applies to this kernel"}
    line["clocks"] = clk

    if not args.no_fp64 and rank == 0:
        order = np.argsort(c["monitoring_points"] * c["path_count"].astype(np.float64))
        sub = c[order[::64]]
        r32 = eng.price_batch(sub, "fp32")
        eng.kernel_timing(reset=True)
        t0 = time.perf_counter()
        r64 = eng.price_batch(sub, "fp64")
        t64 = time.perf_counter() - t0
        k64, _ = eng.kernel_timing(reset=True)
        r32b = eng.price_batch(sub, "fp32")
        k32, _ = eng.kernel_timing(reset=True)
        se = np.maximum(r64["standard_error"], 1e-300)
        err = np.abs(r32["price"] - r64["price"]) / se
        line["fp64_gpu"] = {
            "sample": f"{len(sub)} contracts (every 64th by cost)",
            "fp64_kernel_ms": k64, "fp32_kernel_ms": k32, "speedup_fp32_over_fp64": k64 / k32,
            "fp64_paths_per_second": float(sub["path_count"].astype(np.float64).sum()) / (k64 / 1e3),
            "fp64_path_steps_per_second": path_steps(sub) / (k64 / 1e3),
            "fp32_err_vs_fp64_max_se": float(err.max()), "fp32_err_vs_fp64_mean_se": float(err.mean()),
            "fp64_wall_s": t64}
        assert r32b.tobytes() == r32.tobytes()
    if not args.no_extra and rank == 0:
        line["lsm"] = bench_lsm(eng, peaks)
        line["risk"] = bench_risk(eng, peaks)
        line["heston"] = bench_heston(eng)
        line["qmc"] = bench_qmc(eng, c)
        line["european_1e6"] = bench_european_1e6(eng)
    if not args.no_cpu and rank == 0:
        line["cpu_baseline"] = cpu_baseline_sample(c)
        if "fp64_gpu" in line:
            # like for like: the reference's FP64 arithmetic on the GPU against
            # the same algorithm on the host cores, in path-steps/s
            g = line["fp64_gpu"]["fp64_path_steps_per_second"]
            line["cpu_baseline"]["fp64_gpu_over_cpu"] = g / line["cpu_baseline"]["path_steps_per_s"]
    if rank == 0:
        print(json.dumps(line))
    eng.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
