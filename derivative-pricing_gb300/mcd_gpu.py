"""Python access to libmcd_gpu.so through its C ABI (include/mcd_gpu.h).

Function names and argument order follow the reference's Python module
(bindings/python/src/module.cpp:64-293: ``monte_carlo_european``,
``monte_carlo_asian``, ...), with one extra keyword, ``precision`` ("fp64" for
the reference's arithmetic on the GPU, "fp32" for FP32 paths with FP64
accumulation).  Every call goes to the GPU: there is no CPU fallback, and
loading fails loudly when the library has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
import time as _time
from dataclasses import dataclass

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "build", "libmcd_gpu.so")

u8, i32, u32, u64, dbl, vp = C.c_uint8, C.c_int, C.c_uint32, C.c_uint64, C.c_double, C.c_void_p
P = C.POINTER

CALL, PUT = 0, 1
UP, DOWN = 0, 1
IN, OUT = 0, 1
FIXED, FLOATING = 0, 1
CASH_OR_NOTHING, ASSET_OR_NOTHING = 0, 1
ARITHMETIC, GEOMETRIC = 0, 1
EUROPEAN, DIGITAL, ASIAN, BARRIER, LOOKBACK = 0, 1, 2, 3, 4
FP64, FP32 = 0, 1
SLAB_PATHS = 4096

STATUS = {0: "ok", -1: "invalid argument", -2: "cuda error", -3: "out of memory", -4: "timeout",
          -5: "unsupported", -6: "no device"}


class McResult(C.Structure):
    _fields_ = [("price", dbl), ("standard_error", dbl), ("path_count", u64)]

    def __repr__(self):
        return f"McResult(price={self.price!r}, standard_error={self.standard_error!r}, path_count={self.path_count})"


class HestonParams(C.Structure):
    """mcd_heston_params (= mcd::models::HestonParams, include/mcd/models/heston.hpp:8-18)."""
    _fields_ = [(n, dbl) for n in ("spot", "rate", "carry_yield", "v0", "kappa", "theta", "xi",
                                   "rho", "time")]


class LsmResult(C.Structure):
    """mcd_lsm_result (LsmResult without the policy vectors, plus the inception flag)."""
    _fields_ = [("price", dbl), ("standard_error", dbl), ("path_count", u64),
                ("exercise_at_inception", C.c_int32), ("reserved", C.c_int32)]


LSM_CONTRACT_DTYPE = np.dtype([(n, "<f8") for n in ("spot", "strike", "rate", "carry_yield", "vol",
                                                   "time")] +
                              [("type", "<i4"), ("monitoring_points", "<i4"), ("path_count", "<u8"),
                               ("seed", "<u8")])
LSM_RESULT_DTYPE = np.dtype([("price", "<f8"), ("standard_error", "<f8"), ("path_count", "<u8"),
                             ("exercise_at_inception", "<i4"), ("reserved", "<i4")])
LSM_QR, LSM_MLP = 0, 1
# mcd_american_greeks: price, delta, gamma, vega as (value, standard error), the
# four bumped frozen prices, the bumps, the path count and the inception flag.
AMERICAN_GREEKS_DTYPE = np.dtype([(n, "<f8", (2,)) for n in ("price", "delta", "gamma", "vega")] +
                                 [("scenario", "<f8", (4,)), ("spot_bump", "<f8"), ("vol_bump", "<f8"),
                                  ("path_count", "<u8"), ("exercise_at_inception", "<i4"),
                                  ("reserved", "<i4")])
assert AMERICAN_GREEKS_DTYPE.itemsize == 128
MLP_PARAMS = 4417  # W1[64][2], b1[64], W2[64][64], b2[64], W3[64], b3


def _fptr(a):
    return a.ctypes.data_as(P(C.c_float))


def _regression(r) -> int:
    if r in (0, "qr", "QR", "laguerre"):
        return LSM_QR
    if r in (1, "mlp", "MLP", "learned"):
        return LSM_MLP
    raise ValueError(f"regression must be 'qr' or 'mlp', got {r!r}")


HESTON_DTYPE = np.dtype([(n, "<f8") for n in ("spot", "rate", "carry_yield", "v0", "kappa",
                                              "theta", "xi", "rho", "time")])


class McOptions(C.Structure):
    _fields_ = [("antithetic", u8), ("control_variate", u8), ("brownian_bridge", u8),
                ("reserved", u8), ("num_threads", u32)]


# numpy mirror of mcd_contract (include/mcd_gpu.h), 128 bytes.
CONTRACT_DTYPE = np.dtype([
    ("product", "<i4"), ("type", "<i4"), ("direction", "<i4"), ("knock", "<i4"),
    ("strike_style", "<i4"), ("average_style", "<i4"), ("digital_style", "<i4"),
    ("monitoring_points", "<i4"),
    ("spot", "<f8"), ("strike", "<f8"), ("barrier", "<f8"), ("rebate", "<f8"), ("rate", "<f8"),
    ("carry_yield", "<f8"), ("vol", "<f8"), ("time", "<f8"), ("cash_amount", "<f8"),
    ("path_count", "<u8"), ("seed", "<u8"),
    ("antithetic", "u1"), ("control_variate", "u1"), ("brownian_bridge", "u1"), ("reserved0", "u1"),
    ("reserved1", "<u4"),
])
RESULT_DTYPE = np.dtype([("price", "<f8"), ("standard_error", "<f8"), ("path_count", "<u8")])
assert CONTRACT_DTYPE.itemsize == 128 and RESULT_DTYPE.itemsize == 24


GREEK_NAMES = ("price", "fd_delta", "fd_gamma", "fd_vega", "pathwise_delta", "pathwise_vega",
               "pathwise_rho", "lr_delta", "lr_gamma", "lr_vega", "lr_rho", "lr_theta")
# numpy mirror of mcd_greeks_result: (value, standard_error) per Greek, path count, defined bits.
GREEKS_DTYPE = np.dtype([(n, "<f8", (2,)) for n in GREEK_NAMES] +
                        [("path_count", "<u8"), ("defined", "<u4"), ("reserved", "<u4")])
assert GREEKS_DTYPE.itemsize == 208


class Greek(C.Structure):
    """mcd_greek (= LrGreeksResult / PathwiseGreeksResult)."""
    _fields_ = [("value", dbl), ("standard_error", dbl)]

    def __repr__(self):
        return f"Greek(value={self.value!r}, standard_error={self.standard_error!r})"


class EuropeanGreeks(C.Structure):
    _fields_ = [(n, dbl) for n in ("delta", "gamma", "vega", "theta", "rho")]


class BumpSizes(C.Structure):
    _fields_ = [(n, dbl) for n in ("spot", "vol", "rate", "time")]


class LrGreeks(C.Structure):
    _fields_ = [(n, Greek) for n in ("delta", "gamma", "vega", "rho", "theta")] + \
               [("has_theta", C.c_int32), ("reserved", C.c_int32)]


class PathwiseGreeks(C.Structure):
    _fields_ = [(n, Greek) for n in ("delta", "vega", "rho")]


class McdError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


def _prec(p) -> int:
    if p in (0, "fp64", "FP64", "double"):
        return FP64
    if p in (1, "fp32", "FP32", "float"):
        return FP32
    raise ValueError(f"precision must be 'fp64' or 'fp32', got {p!r}")


_lib = None


def lib():
    """Loads libmcd_gpu.so (raises if it was not built)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} not found: build it with derivative-pricing_gb300/build.py")
    L = C.CDLL(LIB_PATH)

    def sig(name, *args, res=i32):
        f = getattr(L, name)
        f.restype = res
        f.argtypes = list(args)

    D6 = [dbl] * 6
    sig("mcd_abi_version")
    sig("mcd_create", i32, P(vp))
    sig("mcd_destroy", vp, res=None)
    sig("mcd_last_error", vp, res=C.c_char_p)
    sig("mcd_synchronize", vp)
    sig("mcd_price_european", vp, *D6, i32, u64, u64, P(McOptions), i32, P(McResult))
    sig("mcd_price_digital", vp, *D6, i32, i32, dbl, u64, u64, P(McOptions), i32, P(McResult))
    sig("mcd_price_asian", vp, *D6, i32, i32, i32, i32, u64, u64, P(McOptions), i32, P(McResult))
    sig("mcd_price_barrier", vp, *([dbl] * 7), i32, i32, i32, dbl, i32, u64, u64, P(McOptions), i32,
        P(McResult))
    sig("mcd_price_lookback", vp, *D6, i32, i32, i32, u64, u64, P(McOptions), i32, P(McResult))
    sig("mcd_price_batch", vp, vp, C.c_size_t, i32, vp)
    sig("mcd_price_batch_device", vp, vp, C.c_size_t, i32, vp, vp)
    sig("mcd_batch_invalidate", vp)
    sig("mcd_set_launch_shape", vp, i32, i32, i32)
    sig("mcd_get_launch_shape", vp, i32, P(i32), P(i32))
    sig("mcd_autotune", vp, vp, C.c_size_t, i32, P(i32), P(i32), P(dbl))
    sig("mcd_heston_qe_european", vp, P(HestonParams), dbl, i32, i32, u64, u64, i32, P(McResult))
    sig("mcd_heston_qe_batch", vp, vp, C.c_size_t, P(dbl), C.c_size_t, i32, i32, u64, u64, i32, vp)
    sig("mcd_lsm_american", vp, *D6, i32, i32, u64, u64, i32, i32, P(LsmResult), P(dbl), P(u8))
    sig("mcd_lsm_reprice_frozen", vp, *D6, i32, i32, u64, u64, P(dbl), P(u8), i32, i32, P(dbl))
    sig("mcd_lsm_batch", vp, vp, C.c_size_t, i32, i32, vp)
    sig("mcd_lsm_frozen_greeks", vp, *D6, i32, i32, u64, u64, P(dbl), P(u8), i32, dbl, dbl, i32, vp)
    sig("mcd_lsm_greeks_batch", vp, vp, C.c_size_t, dbl, dbl, i32, vp)
    F = P(C.c_float)
    sig("mcd_lsm_set_mlp_config", vp, i32, i32, dbl, dbl)
    sig("mcd_lsm_mlp_policy", vp, C.c_size_t, F, P(u8))
    sig("mcd_lsm_reprice_mlp", vp, *D6, i32, i32, u64, u64, F, P(u8), i32, P(LsmResult))
    sig("mcd_umma_selftest", vp, F, F, F)
    sig("mcd_mlp_gradients", vp, F, F, F, F, F, i32, F, F)
    sig("mcd_mlp_forward", vp, F, F, F, C.c_size_t, F)
    sig("mcd_greeks_batch", vp, vp, C.c_size_t, dbl, dbl, i32, vp)
    sig("mcd_greeks_set_launch_shape", vp, i32, i32, i32)
    sig("mcd_greeks_autotune", vp, vp, C.c_size_t, dbl, dbl, i32, P(i32), P(i32), P(dbl))
    sig("mcd_default_bump_sizes", dbl, dbl, dbl, res=BumpSizes)
    sig("mcd_fd_european", vp, *D6, i32, u64, u64, BumpSizes, i32, P(EuropeanGreeks))
    sig("mcd_lr_european", vp, *D6, i32, u64, u64, i32, P(LrGreeks))
    sig("mcd_lr_digital", vp, *D6, i32, i32, dbl, u64, u64, i32, P(LrGreeks))
    sig("mcd_lr_barrier", vp, *([dbl] * 7), i32, i32, i32, dbl, i32, u64, u64, i32, P(LrGreeks))
    sig("mcd_pathwise_european", vp, *D6, i32, u64, u64, i32, P(PathwiseGreeks))
    sig("mcd_pathwise_asian", vp, *D6, i32, i32, i32, i32, u64, u64, i32, P(PathwiseGreeks))
    sig("mcd_qmc_batch", vp, vp, C.c_size_t, i32, vp)
    sig("mcd_qmc_sobol_european", vp, *D6, i32, u64, i32, P(dbl))
    sig("mcd_qmc_sobol_asian", vp, *D6, i32, i32, i32, u64, i32, P(dbl))
    sig("mcd_sobol_points", vp, C.c_uint, C.c_uint, u64, u64, P(dbl))
    sig("mcd_philox", vp, P(u32), P(u32), C.c_size_t, P(u32))
    sig("mcd_draws", vp, u64, u64, u64, u32, u32, i32, i32, P(dbl))
    sig("mcd_kernel_timing", vp, i32, P(dbl), P(u64))
    sig("mcd_crr_binomial_american", *D6, i32, i32, res=dbl)
    sig("mcd_crr_binomial_bermudan", *D6, i32, i32, i32, res=dbl)
    sig("mcd_crr_binomial", *D6, i32, i32, P(dbl))
    sig("mcd_black_scholes_merton", *D6, i32, res=dbl)
    sig("mcd_black76", *([dbl] * 5), i32, res=dbl)
    sig("mcd_kemna_vorst", *D6, i32, res=dbl)
    sig("mcd_reiner_rubinstein", *([dbl] * 7), i32, i32, i32, dbl, res=dbl)
    sig("mcd_lookback_fixed_strike", *D6, i32, res=dbl)
    sig("mcd_lookback_floating_strike", *([dbl] * 5), i32, res=dbl)
    sig("mcd_digital_analytic", *D6, i32, i32, dbl, res=dbl)
    sig("mcd_forward_price", *([dbl] * 4), res=dbl)
    sig("mcd_forward_value", *([dbl] * 4), res=dbl)
    sig("mcd_futures_mark_to_market", dbl, dbl, res=dbl)
    sig("mcd_heston_semi_analytic", P(HestonParams), dbl, i32, res=dbl)
    _lib = L
    return L


class Engine:
    """One mcd_ctx (device memory, stream, graphs) on one GPU."""

    def __init__(self, device: int = 0):
        self._lib = lib()
        h = vp()
        rc = self._lib.mcd_create(device, C.byref(h))
        if rc != 0:
            raise McdError(rc, self._lib.mcd_last_error(None).decode())
        self.handle = h

    def close(self):
        if getattr(self, "handle", None):
            self._lib.mcd_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != 0:
            raise McdError(rc, self._lib.mcd_last_error(self.handle).decode())

    @staticmethod
    def _opts(antithetic=False, control_variate=False, brownian_bridge=False):
        return McOptions(int(bool(antithetic)), int(bool(control_variate)),
                         int(bool(brownian_bridge)), 0, 1)

    # -- reference pricer signatures (src/pricers/monte_carlo.cpp:233-338) ---------------
    def monte_carlo_european(self, spot, strike, rate, carry_yield, vol, time, type, path_count,
                             seed, antithetic=False, precision="fp64") -> McResult:
        out = McResult()
        o = self._opts(antithetic)
        self._check(self._lib.mcd_price_european(self.handle, spot, strike, rate, carry_yield, vol,
                                                 time, type, path_count, seed, C.byref(o),
                                                 _prec(precision), C.byref(out)))
        return out

    def benchmark_european(self, spot, strike, rate, carry_yield, vol, time, type, path_count, seed,
                           options=None, antithetic=False, precision="fp64") -> dict:
        """The reference's benchmark harness (bindings/python/src/module.cpp:29-60): one
        European pricing call timed on the host clock around the whole call, as a dict.
        ``simd_enabled`` reports the reference's NEON fast path, which this engine does
        not have (the paths run on the GPU)."""
        if options is not None:
            antithetic = bool(options.antithetic)
        t0 = _time.perf_counter()
        r = self.monte_carlo_european(spot, strike, rate, carry_yield, vol, time, type, path_count,
                                      seed, antithetic=antithetic, precision=precision)
        elapsed = _time.perf_counter() - t0
        return {"price": r.price, "standard_error": r.standard_error, "path_count": r.path_count,
                "elapsed_seconds": elapsed,
                "paths_per_second": r.path_count / elapsed if elapsed > 0.0 else 0.0,
                "simd_enabled": False}

    def monte_carlo_digital(self, spot, strike, rate, carry_yield, vol, time, type, style,
                            cash_amount, path_count, seed, antithetic=False,
                            precision="fp64") -> McResult:
        out = McResult()
        o = self._opts(antithetic)
        self._check(self._lib.mcd_price_digital(self.handle, spot, strike, rate, carry_yield, vol,
                                                time, type, style, cash_amount, path_count, seed,
                                                C.byref(o), _prec(precision), C.byref(out)))
        return out

    def monte_carlo_asian(self, spot, strike, rate, carry_yield, vol, time, type, strike_style,
                          average_style, monitoring_points, path_count, seed, antithetic=False,
                          control_variate=False, precision="fp64") -> McResult:
        out = McResult()
        o = self._opts(antithetic, control_variate)
        self._check(self._lib.mcd_price_asian(self.handle, spot, strike, rate, carry_yield, vol,
                                              time, type, strike_style, average_style,
                                              monitoring_points, path_count, seed, C.byref(o),
                                              _prec(precision), C.byref(out)))
        return out

    def monte_carlo_barrier(self, spot, strike, barrier, rate, carry_yield, vol, time, type,
                            direction, knock, rebate, monitoring_points, path_count, seed,
                            antithetic=False, brownian_bridge=False, precision="fp64") -> McResult:
        out = McResult()
        o = self._opts(antithetic, False, brownian_bridge)
        self._check(self._lib.mcd_price_barrier(self.handle, spot, strike, barrier, rate,
                                                carry_yield, vol, time, type, direction, knock,
                                                rebate, monitoring_points, path_count, seed,
                                                C.byref(o), _prec(precision), C.byref(out)))
        return out

    def monte_carlo_lookback(self, spot, strike, rate, carry_yield, vol, time, type, style,
                             monitoring_points, path_count, seed, antithetic=False,
                             precision="fp64") -> McResult:
        out = McResult()
        o = self._opts(antithetic)
        self._check(self._lib.mcd_price_lookback(self.handle, spot, strike, rate, carry_yield, vol,
                                                 time, type, style, monitoring_points, path_count,
                                                 seed, C.byref(o), _prec(precision),
                                                 C.byref(out)))
        return out

    # -- Heston QE (src/pricers/heston.cpp:120-156) -----------------------------------------
    def heston_qe_european(self, params, strike, type, monitoring_points, path_count, seed,
                           precision="fp64") -> McResult:
        p = params if isinstance(params, HestonParams) else HestonParams(*params)
        out = McResult()
        self._check(self._lib.mcd_heston_qe_european(self.handle, C.byref(p), strike, type,
                                                     monitoring_points, path_count, seed,
                                                     _prec(precision), C.byref(out)))
        return out

    def heston_qe_batch(self, sets, strikes, type, monitoring_points, path_count, seed,
                        precision="fp32") -> np.ndarray:
        """sets: array of HESTON_DTYPE records (or n x 9 floats); returns n_sets x n_strikes."""
        sets = np.ascontiguousarray(sets, dtype=np.float64).reshape(-1, 9) \
            if not (isinstance(sets, np.ndarray) and sets.dtype == HESTON_DTYPE) \
            else np.ascontiguousarray(sets)
        strikes = np.ascontiguousarray(strikes, dtype=np.float64)
        out = np.zeros((len(sets), len(strikes)), dtype=RESULT_DTYPE)
        self._check(self._lib.mcd_heston_qe_batch(self.handle, sets.ctypes.data, len(sets),
                                                  strikes.ctypes.data_as(P(dbl)), len(strikes),
                                                  type, monitoring_points, path_count, seed,
                                                  _prec(precision), out.ctypes.data))
        return out

    # -- Longstaff-Schwartz (src/pricers/lsm.cpp:62-213) -------------------------------------
    def monte_carlo_lsm_american(self, spot, strike, rate, carry_yield, vol, time, type,
                                 monitoring_points, path_count, seed, precision="fp64",
                                 regression="qr", policy=False):
        """Returns an LsmResult, or (LsmResult, coefficients[(n+1), 4], has[n+1]) with policy=True."""
        out = LsmResult()
        n1 = monitoring_points + 1
        co = np.zeros((n1, 4), dtype=np.float64) if policy else None
        ha = np.zeros(n1, dtype=np.uint8) if policy else None
        self._check(self._lib.mcd_lsm_american(
            self.handle, spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
            path_count, seed, _prec(precision), _regression(regression), C.byref(out),
            co.ctypes.data_as(P(dbl)) if policy else None,
            ha.ctypes.data_as(P(u8)) if policy else None))
        return (out, co, ha) if policy else out

    def reprice_against_frozen_policy(self, spot, strike, rate, carry_yield, vol, time, type,
                                      monitoring_points, path_count, seed, coefficients, has,
                                      exercise_at_inception=False, precision="fp64") -> float:
        co = np.ascontiguousarray(coefficients, dtype=np.float64)
        ha = np.ascontiguousarray(has, dtype=np.uint8)
        price = dbl()
        self._check(self._lib.mcd_lsm_reprice_frozen(
            self.handle, spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
            path_count, seed, co.ctypes.data_as(P(dbl)), ha.ctypes.data_as(P(u8)),
            int(bool(exercise_at_inception)), _prec(precision), C.byref(price)))
        return price.value

    def lsm_batch(self, contracts, precision="fp32", regression="qr") -> np.ndarray:
        contracts = np.ascontiguousarray(contracts, dtype=LSM_CONTRACT_DTYPE)
        out = np.zeros(len(contracts), dtype=LSM_RESULT_DTYPE)
        self._check(self._lib.mcd_lsm_batch(self.handle, contracts.ctypes.data, len(contracts),
                                            _prec(precision), _regression(regression),
                                            out.ctypes.data))
        return out

    def lsm_frozen_greeks(self, spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
                          path_count, seed, coefficients, has, exercise_at_inception=False,
                          spot_bump=None, vol_bump=None, precision="fp64") -> np.record:
        """Delta, gamma and vega of an American option against its frozen QR policy
        (mcd_lsm_frozen_greeks); bumps default to 1% of spot and of vol."""
        co = np.ascontiguousarray(coefficients, dtype=np.float64)
        ha = np.ascontiguousarray(has, dtype=np.uint8)
        out = np.zeros(1, dtype=AMERICAN_GREEKS_DTYPE)
        self._check(self._lib.mcd_lsm_frozen_greeks(
            self.handle, spot, strike, rate, carry_yield, vol, time, type, monitoring_points, path_count,
            seed, co.ctypes.data_as(P(dbl)), ha.ctypes.data_as(P(u8)), int(bool(exercise_at_inception)),
            0.01 * spot if spot_bump is None else spot_bump, 0.01 * vol if vol_bump is None else vol_bump,
            _prec(precision), out.ctypes.data))
        return out[0]

    def lsm_greeks_batch(self, contracts, spot_bump_rel=0.01, vol_bump_rel=0.01,
                         precision="fp32") -> np.ndarray:
        """Fits every contract's policy and returns its frozen-boundary Greeks
        (mcd_lsm_greeks_batch) as an AMERICAN_GREEKS_DTYPE array."""
        contracts = np.ascontiguousarray(contracts, dtype=LSM_CONTRACT_DTYPE)
        out = np.zeros(len(contracts), dtype=AMERICAN_GREEKS_DTYPE)
        self._check(self._lib.mcd_lsm_greeks_batch(self.handle, contracts.ctypes.data, len(contracts),
                                                   spot_bump_rel, vol_bump_rel, _prec(precision),
                                                   out.ctypes.data))
        return out

    # -- learned regression ----------------------------------------------------------------
    def set_mlp_config(self, steps_first=100, steps=0, lr_first=3e-3, lr=1e-3):
        """Training schedule of the learned regression (see mcd_lsm_set_mlp_config)."""
        self._check(self._lib.mcd_lsm_set_mlp_config(self.handle, steps_first, steps, lr_first, lr))

    def mlp_policy(self, contract: int, monitoring_points: int):
        w = np.zeros((monitoring_points + 1, MLP_PARAMS), dtype=np.float32)
        has = np.zeros(monitoring_points + 1, dtype=np.uint8)
        self._check(self._lib.mcd_lsm_mlp_policy(self.handle, contract, _fptr(w),
                                                 has.ctypes.data_as(P(u8))))
        return w, has

    def reprice_mlp(self, spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
                    path_count, seed, weights, has, precision="fp32") -> LsmResult:
        w = np.ascontiguousarray(weights, dtype=np.float32)
        h = np.ascontiguousarray(has, dtype=np.uint8)
        out = LsmResult()
        self._check(self._lib.mcd_lsm_reprice_mlp(self.handle, spot, strike, rate, carry_yield, vol,
                                                  time, type, monitoring_points, path_count, seed,
                                                  _fptr(w), h.ctypes.data_as(P(u8)),
                                                  _prec(precision), C.byref(out)))
        return out

    def umma_selftest(self, a, b):
        a = np.ascontiguousarray(a, dtype=np.float32).reshape(128, 64)
        b = np.ascontiguousarray(b, dtype=np.float32).reshape(64, 64)
        d = np.zeros((128, 64), dtype=np.float32)
        self._check(self._lib.mcd_umma_selftest(self.handle, _fptr(a), _fptr(b), _fptr(d)))
        return d

    def mlp_gradients(self, params, x0, x1, y, w):
        params = np.ascontiguousarray(params, dtype=np.float32)
        arrs = [np.ascontiguousarray(v, dtype=np.float32) for v in (x0, x1, y, w)]
        g = np.zeros(MLP_PARAMS, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        self._check(self._lib.mcd_mlp_gradients(self.handle, _fptr(params), *[_fptr(a) for a in arrs],
                                                len(arrs[0]), _fptr(g), _fptr(loss)))
        return g, float(loss[0])

    def mlp_forward(self, params, x0, x1):
        params = np.ascontiguousarray(params, dtype=np.float32)
        x0 = np.ascontiguousarray(x0, dtype=np.float32)
        x1 = np.ascontiguousarray(x1, dtype=np.float32)
        out = np.zeros(len(x0), dtype=np.float32)
        self._check(self._lib.mcd_mlp_forward(self.handle, _fptr(params), _fptr(x0), _fptr(x1),
                                              len(x0), _fptr(out)))
        return out

    # -- batch -----------------------------------------------------------------------------
    def price_batch(self, contracts: np.ndarray, precision="fp64") -> np.ndarray:
        contracts = np.ascontiguousarray(contracts, dtype=CONTRACT_DTYPE)
        out = np.zeros(len(contracts), dtype=RESULT_DTYPE)
        self._check(self._lib.mcd_price_batch(self.handle, contracts.ctypes.data, len(contracts),
                                              _prec(precision), out.ctypes.data))
        return out

    def price_batch_device(self, contracts_ptr: int, n: int, results_ptr: int, precision="fp32",
                           stream: int = 0) -> None:
        self._check(self._lib.mcd_price_batch_device(self.handle, vp(contracts_ptr), n,
                                                     _prec(precision), vp(results_ptr),
                                                     vp(stream) if stream else None))

    def invalidate(self):
        self._check(self._lib.mcd_batch_invalidate(self.handle))

    def set_launch_shape(self, precision, variant: int, ctas_per_sm: int):
        self._check(self._lib.mcd_set_launch_shape(self.handle, _prec(precision), variant,
                                                   ctas_per_sm))

    def launch_shape(self, precision):
        v, c = i32(), i32()
        self._check(self._lib.mcd_get_launch_shape(self.handle, _prec(precision), C.byref(v),
                                                   C.byref(c)))
        return v.value, c.value

    def autotune(self, contracts: np.ndarray, precision="fp32"):
        contracts = np.ascontiguousarray(contracts, dtype=CONTRACT_DTYPE)
        v, c, ms = i32(), i32(), dbl()
        self._check(self._lib.mcd_autotune(self.handle, contracts.ctypes.data, len(contracts),
                                           _prec(precision), C.byref(v), C.byref(c), C.byref(ms)))
        return v.value, c.value, ms.value

    def synchronize(self):
        self._check(self._lib.mcd_synchronize(self.handle))

    def kernel_timing(self, reset=False):
        ms, n = dbl(), u64()
        self._check(self._lib.mcd_kernel_timing(self.handle, int(reset), C.byref(ms), C.byref(n)))
        return ms.value, n.value

    # -- draws -----------------------------------------------------------------------------
    # -- Greeks ----------------------------------------------------------------------------
    def greeks_batch(self, contracts: np.ndarray, spot_bump_rel=1e-4, vol_bump_rel=1e-4,
                     precision="fp32") -> np.ndarray:
        """Price, CRN finite-difference, pathwise and likelihood-ratio Greeks of every contract
        in one launch (mcd_greeks_batch); returns a GREEKS_DTYPE array."""
        contracts = np.ascontiguousarray(contracts, dtype=CONTRACT_DTYPE)
        out = np.zeros(len(contracts), dtype=GREEKS_DTYPE)
        self._check(self._lib.mcd_greeks_batch(self.handle, contracts.ctypes.data, len(contracts),
                                               spot_bump_rel, vol_bump_rel, _prec(precision),
                                               out.ctypes.data))
        return out

    def set_greeks_launch_shape(self, precision, variant: int, ctas_per_sm: int):
        self._check(self._lib.mcd_greeks_set_launch_shape(self.handle, _prec(precision), variant,
                                                          ctas_per_sm))

    def greeks_autotune(self, contracts: np.ndarray, spot_bump_rel=1e-4, vol_bump_rel=1e-4,
                        precision="fp32"):
        contracts = np.ascontiguousarray(contracts, dtype=CONTRACT_DTYPE)
        v, c, ms = i32(), i32(), dbl()
        self._check(self._lib.mcd_greeks_autotune(self.handle, contracts.ctypes.data, len(contracts),
                                                  spot_bump_rel, vol_bump_rel, _prec(precision),
                                                  C.byref(v), C.byref(c), C.byref(ms)))
        return v.value, c.value, ms.value

    def default_bump_sizes(self, spot, vol, time) -> BumpSizes:
        return self._lib.mcd_default_bump_sizes(spot, vol, time)

    def finite_difference_european(self, spot, strike, rate, carry_yield, vol, time, type,
                                   path_count, seed, bumps=None, precision="fp64") -> EuropeanGreeks:
        b = bumps if bumps is not None else self.default_bump_sizes(spot, vol, time)
        out = EuropeanGreeks()
        self._check(self._lib.mcd_fd_european(self.handle, spot, strike, rate, carry_yield, vol, time,
                                              type, path_count, seed, b, _prec(precision),
                                              C.byref(out)))
        return out

    def likelihood_ratio_european(self, spot, strike, rate, carry_yield, vol, time, type,
                                  path_count, seed, precision="fp64") -> LrGreeks:
        out = LrGreeks()
        self._check(self._lib.mcd_lr_european(self.handle, spot, strike, rate, carry_yield, vol, time,
                                              type, path_count, seed, _prec(precision), C.byref(out)))
        return out

    def likelihood_ratio_digital(self, spot, strike, rate, carry_yield, vol, time, type, style,
                                 cash_amount, path_count, seed, precision="fp64") -> LrGreeks:
        out = LrGreeks()
        self._check(self._lib.mcd_lr_digital(self.handle, spot, strike, rate, carry_yield, vol, time,
                                             type, style, cash_amount, path_count, seed,
                                             _prec(precision), C.byref(out)))
        return out

    def likelihood_ratio_barrier(self, spot, strike, barrier, rate, carry_yield, vol, time, type,
                                 direction, knock, rebate, monitoring_points, path_count, seed,
                                 precision="fp64") -> LrGreeks:
        out = LrGreeks()
        self._check(self._lib.mcd_lr_barrier(self.handle, spot, strike, barrier, rate, carry_yield, vol,
                                             time, type, direction, knock, rebate, monitoring_points,
                                             path_count, seed, _prec(precision), C.byref(out)))
        return out

    def pathwise_european(self, spot, strike, rate, carry_yield, vol, time, type, path_count, seed,
                          precision="fp64") -> PathwiseGreeks:
        out = PathwiseGreeks()
        self._check(self._lib.mcd_pathwise_european(self.handle, spot, strike, rate, carry_yield, vol,
                                                    time, type, path_count, seed, _prec(precision),
                                                    C.byref(out)))
        return out

    def pathwise_asian(self, spot, strike, rate, carry_yield, vol, time, type, strike_style,
                       average_style, monitoring_points, path_count, seed,
                       precision="fp64") -> PathwiseGreeks:
        out = PathwiseGreeks()
        self._check(self._lib.mcd_pathwise_asian(self.handle, spot, strike, rate, carry_yield, vol,
                                                 time, type, strike_style, average_style,
                                                 monitoring_points, path_count, seed,
                                                 _prec(precision), C.byref(out)))
        return out

    # -- Sobol quasi-Monte Carlo ------------------------------------------------------------
    def qmc_batch(self, contracts: np.ndarray, precision="fp64") -> np.ndarray:
        """QMC prices (Sobol + Brownian bridge) of a batch; standard_error is 0."""
        contracts = np.ascontiguousarray(contracts, dtype=CONTRACT_DTYPE)
        out = np.zeros(len(contracts), dtype=RESULT_DTYPE)
        self._check(self._lib.mcd_qmc_batch(self.handle, contracts.ctypes.data, len(contracts),
                                            _prec(precision), out.ctypes.data))
        return out

    def qmc_sobol_european(self, spot, strike, rate, carry_yield, vol, time, type, path_count,
                           precision="fp64") -> float:
        p = dbl()
        self._check(self._lib.mcd_qmc_sobol_european(self.handle, spot, strike, rate, carry_yield, vol,
                                                     time, type, path_count, _prec(precision),
                                                     C.byref(p)))
        return p.value

    def qmc_sobol_asian(self, spot, strike, rate, carry_yield, vol, time, type, strike_style,
                        monitoring_points, path_count, precision="fp64") -> float:
        p = dbl()
        self._check(self._lib.mcd_qmc_sobol_asian(self.handle, spot, strike, rate, carry_yield, vol,
                                                  time, type, strike_style, monitoring_points,
                                                  path_count, _prec(precision), C.byref(p)))
        return p.value

    def sobol_points(self, dim_begin, n_dims, index_begin, n_indices) -> np.ndarray:
        out = np.zeros((n_indices, n_dims), dtype=np.float64)
        self._check(self._lib.mcd_sobol_points(self.handle, dim_begin, n_dims, index_begin, n_indices,
                                               out.ctypes.data_as(P(dbl))))
        return out

    def philox(self, counters: np.ndarray, keys: np.ndarray) -> np.ndarray:
        counters = np.ascontiguousarray(counters, dtype=np.uint32).reshape(-1, 4)
        keys = np.ascontiguousarray(keys, dtype=np.uint32).reshape(-1, 2)
        out = np.zeros_like(counters)
        self._check(self._lib.mcd_philox(self.handle, counters.ctypes.data_as(P(u32)),
                                         keys.ctypes.data_as(P(u32)), len(counters),
                                         out.ctypes.data_as(P(u32))))
        return out

    def draws(self, seed, path_begin, n_paths, draw_begin, n_draws, stream_id=0,
              precision="fp64") -> np.ndarray:
        out = np.zeros((n_paths, n_draws), dtype=np.float64)
        self._check(self._lib.mcd_draws(self.handle, seed, path_begin, n_paths, draw_begin, n_draws,
                                        stream_id, _prec(precision), out.ctypes.data_as(P(dbl))))
        return out


# -- closed forms and lattices (host FP64 in libmcd_gpu.so; module.cpp:179-198, 284) -----
@dataclass
class BinomialResult:
    """mcd::pricers::BinomialResult (include/mcd/pricers/binomial.hpp)."""
    price: float
    risk_neutral_probability: float
    up_factor: float
    down_factor: float


def black_scholes_merton(spot, strike, rate, carry_yield, vol, time, type) -> float:
    return lib().mcd_black_scholes_merton(spot, strike, rate, carry_yield, vol, time, int(type))


def black76(forward, strike, rate, vol, time, type) -> float:
    return lib().mcd_black76(forward, strike, rate, vol, time, int(type))


def kemna_vorst(spot, strike, rate, carry_yield, vol, time, type) -> float:
    return lib().mcd_kemna_vorst(spot, strike, rate, carry_yield, vol, time, int(type))


def reiner_rubinstein(spot, strike, barrier, rate, carry_yield, vol, time, type, direction, knock,
                      rebate=0.0) -> float:
    return lib().mcd_reiner_rubinstein(spot, strike, barrier, rate, carry_yield, vol, time, int(type),
                                       int(direction), int(knock), rebate)


def lookback_fixed_strike(spot, strike, rate, carry_yield, vol, time, type) -> float:
    return lib().mcd_lookback_fixed_strike(spot, strike, rate, carry_yield, vol, time, int(type))


def lookback_floating_strike(spot, rate, carry_yield, vol, time, type) -> float:
    return lib().mcd_lookback_floating_strike(spot, rate, carry_yield, vol, time, int(type))


def digital(spot, strike, rate, carry_yield, vol, time, type, style, cash_amount=1.0) -> float:
    return lib().mcd_digital_analytic(spot, strike, rate, carry_yield, vol, time, int(type), int(style),
                                      cash_amount)


def forward_price(spot, rate, carry_yield, time) -> float:
    return lib().mcd_forward_price(spot, rate, carry_yield, time)


def forward_value(forward_now, forward_at_inception, rate, time_to_expiry) -> float:
    return lib().mcd_forward_value(forward_now, forward_at_inception, rate, time_to_expiry)


def futures_mark_to_market(futures_price_new, futures_price_old) -> float:
    return lib().mcd_futures_mark_to_market(futures_price_new, futures_price_old)


def crr_binomial(spot, strike, rate, carry_yield, vol, time, steps, type) -> BinomialResult:
    out = (dbl * 4)()
    rc = lib().mcd_crr_binomial(spot, strike, rate, carry_yield, vol, time, steps, int(type), out)
    if rc != 0:
        raise McdError(rc, "crr_binomial: steps must be >= 1")
    return BinomialResult(*out)


def crr_binomial_bermudan(spot, strike, rate, carry_yield, vol, time, exercise_dates, steps_per_date,
                          type) -> float:
    """Bermudan CRR price, exercise at the LSM dates (mcd_crr_binomial_bermudan)."""
    return lib().mcd_crr_binomial_bermudan(spot, strike, rate, carry_yield, vol, time, int(exercise_dates),
                                           int(steps_per_date), int(type))


def crr_binomial_american(spot, strike, rate, carry_yield, vol, time, steps, type) -> float:
    """Cox-Ross-Rubinstein American price."""
    return lib().mcd_crr_binomial_american(spot, strike, rate, carry_yield, vol, time, steps, int(type))


def heston_semi_analytic(params: HestonParams, strike, type) -> float:
    return lib().mcd_heston_semi_analytic(C.byref(params), strike, int(type))


def contracts(n: int) -> np.ndarray:
    """A zeroed contract array (cash_amount 1, monitoring_points 1)."""
    a = np.zeros(n, dtype=CONTRACT_DTYPE)
    a["cash_amount"] = 1.0
    a["monitoring_points"] = 1
    return a
