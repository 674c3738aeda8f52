"""ctypes loader for the CPU oracle (test infrastructure only).

Loads ``oracle/build/libmcd_oracle.so`` (the C restatement of the reference's
hot path, see mcd_oracle.h) and, where it was built, ``oracle/_ref/libmcd_ref.so``
(the reference compiled from its own sources).  Only the tests, the smoke check
and the benchmark's CPU-baseline leg import this module; the product library
never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "build", "libmcd_oracle.so")
REF_SO = os.path.join(HERE, "_ref", "libmcd_ref.so")

u8, i32, u32, u64, dbl = C.c_uint8, C.c_int, C.c_uint32, C.c_uint64, C.c_double
P = C.POINTER


class McResult(C.Structure):
    _fields_ = [("price", dbl), ("standard_error", dbl), ("path_count", u64)]


class Options(C.Structure):
    _fields_ = [("antithetic", i32), ("control_variate", i32), ("brownian_bridge", i32),
                ("num_threads", C.c_uint), ("chunk_count", C.c_uint)]


class HestonParams(C.Structure):
    _fields_ = [(n, dbl) for n in ("spot", "rate", "carry_yield", "v0", "kappa", "theta", "xi",
                                   "rho", "time")]


class EuropeanGreeks(C.Structure):
    _fields_ = [(n, dbl) for n in ("delta", "gamma", "vega", "theta", "rho")]


class Bumps(C.Structure):
    _fields_ = [(n, dbl) for n in ("spot", "vol", "rate", "time")]


class Greek(C.Structure):
    _fields_ = [("value", dbl), ("standard_error", dbl)]


class LrGreeks(C.Structure):
    _fields_ = [("delta", Greek), ("gamma", Greek), ("vega", Greek), ("rho", Greek),
                ("theta", Greek), ("has_theta", i32)]


class PathwiseGreeks(C.Structure):
    _fields_ = [("delta", Greek), ("vega", Greek), ("rho", Greek)]


class Contract(C.Structure):
    """Same layout as mcd_contract in include/mcd_gpu.h."""
    _fields_ = [(n, C.c_int32) for n in ("product", "type", "direction", "knock", "strike_style",
                                         "average_style", "digital_style", "monitoring_points")] + \
               [(n, dbl) for n in ("spot", "strike", "barrier", "rebate", "rate", "carry_yield",
                                   "vol", "time", "cash_amount")] + \
               [("path_count", u64), ("seed", u64), ("antithetic", u8), ("control_variate", u8),
                ("brownian_bridge", u8), ("reserved0", u8), ("reserved1", u32)]


def build(force: bool = False) -> None:
    """Compile the C restatement (and the reference, when its sources exist)."""
    targets = ["oracle", "ref-if-present"]  # the Makefile knows where the reference lies
    subprocess.run(["make", "-s", "-C", HERE] + (["-B"] if force else []) + targets, check=True)


def _sig(lib, name, res, *args):
    f = getattr(lib, name)
    f.restype = res
    f.argtypes = list(args)
    return f


def load():
    if not os.path.exists(ORACLE_SO):
        build()
    lib = C.CDLL(ORACLE_SO)
    D7 = [dbl] * 6 + [i32]
    _sig(lib, "orc_philox4x32_10", None, P(u32), P(u32), P(u32))
    _sig(lib, "orc_uniform_open01", dbl, u32)
    _sig(lib, "orc_normal_cdf", dbl, dbl)
    _sig(lib, "orc_normal_pdf", dbl, dbl)
    _sig(lib, "orc_inv_normal_cdf", dbl, dbl)
    _sig(lib, "orc_normal_variate", dbl, u64, u64, u32)
    _sig(lib, "orc_uniform_variate", dbl, u64, u64, u32)
    _sig(lib, "orc_default_chunk_count", C.c_uint)
    _sig(lib, "orc_sobol_point", dbl, C.c_uint, u64)
    _sig(lib, "orc_sobol_bits", u32, C.c_uint, u64)
    _sig(lib, "orc_sobol_directions", None, C.c_uint, P(u32))
    _sig(lib, "orc_sobol_polynomial", i32, C.c_uint, P(C.c_uint), P(u32))
    _sig(lib, "orc_brownian_bridge_gbm_path", None, dbl, dbl, dbl, dbl, dbl, i32, P(dbl), P(dbl))
    _sig(lib, "orc_mc_european", McResult, *D7, u64, u64, P(Options))
    _sig(lib, "orc_mc_digital", McResult, *D7, i32, dbl, u64, u64, P(Options))
    _sig(lib, "orc_mc_asian", McResult, *D7, i32, i32, i32, u64, u64, P(Options))
    _sig(lib, "orc_mc_barrier", McResult, dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, i32, i32, dbl,
         i32, u64, u64, P(Options))
    _sig(lib, "orc_mc_lookback", McResult, *D7, i32, i32, u64, u64, P(Options))
    _sig(lib, "orc_lsm_american", McResult, *D7, i32, u64, u64, P(dbl), P(u8), P(i32))
    _sig(lib, "orc_lsm_reprice_frozen", dbl, *D7, i32, u64, u64, P(dbl), P(u8), i32)
    _sig(lib, "orc_laguerre_basis", None, dbl, P(dbl))
    _sig(lib, "orc_householder_least_squares", None, P(dbl), i32, i32, P(dbl), P(dbl))
    _sig(lib, "orc_heston_qe_european", McResult, P(HestonParams), dbl, i32, i32, u64, u64)
    _sig(lib, "orc_heston_semi_analytic", dbl, P(HestonParams), dbl, i32)
    _sig(lib, "orc_qmc_sobol_european", dbl, *D7, u64)
    _sig(lib, "orc_qmc_sobol_asian", dbl, *D7, i32, i32, u64)
    _sig(lib, "orc_default_bump_sizes", Bumps, dbl, dbl, dbl)
    _sig(lib, "orc_fd_european", EuropeanGreeks, *D7, u64, u64, Bumps, C.c_uint)
    _sig(lib, "orc_lr_european", LrGreeks, *D7, u64, u64)
    _sig(lib, "orc_lr_digital", LrGreeks, *D7, i32, dbl, u64, u64)
    _sig(lib, "orc_lr_barrier", LrGreeks, dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, i32, i32, dbl,
         i32, u64, u64)
    _sig(lib, "orc_pathwise_european", PathwiseGreeks, *D7, u64, u64)
    _sig(lib, "orc_pathwise_asian", PathwiseGreeks, *D7, i32, i32, i32, u64, u64)
    _sig(lib, "orc_bsm", dbl, *D7)
    _sig(lib, "orc_kemna_vorst", dbl, *D7)
    _sig(lib, "orc_reiner_rubinstein", dbl, dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, i32, i32, dbl)
    _sig(lib, "orc_lookback_fixed", dbl, *D7)
    _sig(lib, "orc_lookback_floating", dbl, dbl, dbl, dbl, dbl, dbl, i32)
    _sig(lib, "orc_digital_analytic", dbl, *D7, i32, dbl)
    _sig(lib, "orc_crr_binomial_american", dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, i32)
    _sig(lib, "orc_price_batch", None, P(Contract), i32, C.c_uint, C.c_uint, P(McResult))
    _sig(lib, "orc_heston_batch", None, P(HestonParams), i32, P(dbl), i32, i32, i32, u64, u64,
         C.c_uint, P(McResult))
    _sig(lib, "orc_lsm_batch", None, P(dbl), i32, i32, u64, u64, C.c_uint, P(McResult))
    return lib


def load_ref():
    """The reference compiled from source, or None where it was not built."""
    if not os.path.exists(REF_SO):
        return None
    lib = C.CDLL(REF_SO)
    D7 = [dbl] * 6 + [i32]
    _sig(lib, "ref_logical_chunk_count", C.c_uint)
    _sig(lib, "ref_philox", None, P(u32), P(u32), P(u32))
    _sig(lib, "ref_normal_variate", dbl, u64, u64, u32)
    _sig(lib, "ref_uniform_variate", dbl, u64, u64, u32)
    _sig(lib, "ref_inv_normal_cdf", dbl, dbl)
    _sig(lib, "ref_normal_cdf", dbl, dbl)
    _sig(lib, "ref_sobol_point", dbl, C.c_uint, u64)
    _sig(lib, "ref_brownian_bridge_gbm_path", None, dbl, dbl, dbl, dbl, dbl, i32, P(dbl), P(dbl))
    _sig(lib, "ref_mc_european", None, *D7, u64, u64, i32, C.c_uint, P(dbl))
    _sig(lib, "ref_mc_digital", None, *D7, i32, dbl, u64, u64, i32, C.c_uint, P(dbl))
    _sig(lib, "ref_mc_asian", None, *D7, i32, i32, i32, u64, u64, i32, i32, C.c_uint, P(dbl))
    _sig(lib, "ref_mc_barrier", None, dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, i32, i32, dbl, i32,
         u64, u64, i32, i32, C.c_uint, P(dbl))
    _sig(lib, "ref_mc_lookback", None, *D7, i32, i32, u64, u64, i32, C.c_uint, P(dbl))
    _sig(lib, "ref_lsm_american", None, *D7, i32, u64, u64, P(dbl), P(dbl), P(u8), P(i32))
    _sig(lib, "ref_lsm_reprice_frozen", dbl, *D7, i32, u64, u64, P(dbl), P(u8), i32)
    _sig(lib, "ref_heston_qe", None, P(dbl), dbl, i32, i32, u64, u64, P(dbl))
    _sig(lib, "ref_heston_semi_analytic", dbl, P(dbl), dbl, i32)
    _sig(lib, "ref_qmc_european", dbl, *D7, u64)
    _sig(lib, "ref_qmc_asian", dbl, *D7, i32, i32, u64)
    _sig(lib, "ref_fd_european", None, *D7, u64, u64, P(dbl), P(dbl))
    _sig(lib, "ref_default_bumps", None, dbl, dbl, dbl, P(dbl))
    _sig(lib, "ref_lr_european", i32, *D7, u64, u64, P(dbl))
    _sig(lib, "ref_lr_digital", i32, *D7, i32, dbl, u64, u64, P(dbl))
    _sig(lib, "ref_lr_barrier", i32, dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, i32, i32, dbl, i32,
         u64, u64, P(dbl))
    _sig(lib, "ref_pathwise_european", None, *D7, u64, u64, P(dbl))
    _sig(lib, "ref_pathwise_asian", None, *D7, i32, i32, i32, u64, u64, P(dbl))
    _sig(lib, "ref_bsm", dbl, *D7)
    _sig(lib, "ref_kemna_vorst", dbl, *D7)
    _sig(lib, "ref_reiner_rubinstein", dbl, dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, i32, i32, dbl)
    _sig(lib, "ref_lookback_fixed", dbl, *D7)
    _sig(lib, "ref_lookback_floating", dbl, dbl, dbl, dbl, dbl, dbl, i32)
    _sig(lib, "ref_digital_analytic", dbl, *D7, i32, dbl)
    _sig(lib, "ref_crr_american", dbl, dbl, dbl, dbl, dbl, dbl, dbl, i32, i32)
    return lib


def options(antithetic=False, control_variate=False, brownian_bridge=False, num_threads=1,
            chunk_count=0) -> Options:
    return Options(int(antithetic), int(control_variate), int(brownian_bridge), num_threads,
                   chunk_count)


def dbuf(n):
    return (dbl * n)()
