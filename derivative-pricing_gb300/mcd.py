"""``mcd``: the reference's Python module (bindings/python/src/module.cpp:64-293),
same names, argument order, defaults, enums and result attributes, over the GPU
engine's C ABI.  Code written against the reference module runs unchanged with
this directory on ``sys.path``.

What differs, because a GPU sits underneath:

* every Monte Carlo call runs on the GPU (FP64 arithmetic by default, the
  reference's; ``set_precision("fp32")`` switches the calling thread to FP32
  paths with FP64 accumulation);
* calls take an engine context (device ``MCD_GPU_DEVICE``, default 0) from a pool
  of warmed contexts (``MCD_GPU_POOL``, default 2, more on demand), so calls from
  several threads run concurrently; ctypes releases the GIL around every foreign
  call, as the reference's ``gil_scoped_release`` does;
* ``McOptions.num_threads`` is accepted and ignored (the path loop is on the GPU);
* ``HAS_NEON`` is False: the reference's NEON batch path does not exist here,
  and ``benchmark_european`` reports ``simd_enabled`` accordingly;
* ``SOBOL_MAX_DIMENSIONS`` is 256 (the reference stops at 7).

The closed forms and lattices are host FP64 functions of the same library.
"""
from __future__ import annotations

import enum
import os
import threading

import mcd_gpu as _g

# -- enums (include/mcd/core/types.hpp:12-17) -------------------------------------


class OptionType(enum.IntEnum):
    Call = 0
    Put = 1


class BarrierDirection(enum.IntEnum):
    Up = 0
    Down = 1


class BarrierKnock(enum.IntEnum):
    In = 0
    Out = 1


class StrikeStyle(enum.IntEnum):
    Fixed = 0
    Floating = 1


class DigitalStyle(enum.IntEnum):
    CashOrNothing = 0
    AssetOrNothing = 1


class AverageStyle(enum.IntEnum):
    Arithmetic = 0
    Geometric = 1


SOBOL_MAX_DIMENSIONS = 256
HAS_NEON = False

# -- value types ------------------------------------------------------------------


class McOptions:
    """mcd::pricers::McOptions (include/mcd/pricers/monte_carlo.hpp:18-33)."""

    def __init__(self, antithetic=False, control_variate=False, brownian_bridge=False, num_threads=1):
        self.antithetic = antithetic
        self.control_variate = control_variate
        self.brownian_bridge = brownian_bridge
        self.num_threads = num_threads


HestonParams = _g.HestonParams
BinomialResult = _g.BinomialResult
McResult = _g.McResult
BumpSizes = _g.BumpSizes
EuropeanGreeks = _g.EuropeanGreeks


class _Result:
    __slots__ = ()

    def __repr__(self):
        body = ", ".join(f"{k}={getattr(self, k)!r}" for k in self.__slots__)
        return f"{type(self).__name__}({body})"


class LrGreeksResult(_Result):
    __slots__ = ("value", "standard_error")

    def __init__(self, value, standard_error):
        self.value, self.standard_error = value, standard_error


PathwiseGreeksResult = LrGreeksResult


class LrGreeks(_Result):
    """delta, gamma, vega, rho; theta is None for the barrier (likelihood_ratio.cpp:105-154)."""
    __slots__ = ("delta", "gamma", "vega", "rho", "theta")

    def __init__(self, raw):
        for n in ("delta", "gamma", "vega", "rho"):
            g = getattr(raw, n)
            setattr(self, n, LrGreeksResult(g.value, g.standard_error))
        self.theta = LrGreeksResult(raw.theta.value, raw.theta.standard_error) if raw.has_theta else None


class PathwiseGreeks(_Result):
    """delta, vega, rho only: gamma and theta are undefined for pathwise estimators."""
    __slots__ = ("delta", "vega", "rho")

    def __init__(self, raw):
        for n in self.__slots__:
            g = getattr(raw, n)
            setattr(self, n, PathwiseGreeksResult(g.value, g.standard_error))


class QmcResult(_Result):
    """A deterministic Sobol estimate: a price, no standard error."""
    __slots__ = ("price",)

    def __init__(self, price):
        self.price = price


class LsmResult(_Result):
    __slots__ = ("price", "standard_error")

    def __init__(self, price, standard_error):
        self.price, self.standard_error = price, standard_error


HestonMcResult = McResult

# -- engine pool ------------------------------------------------------------------
# A context serves one call at a time; a call takes an idle context from the pool
# (creating one when every context is busy) and returns it afterwards, so calls
# from several threads run concurrently, and threads that come and go reuse the
# contexts (and the graphs captured in them) of earlier ones.  The first call
# creates MCD_GPU_POOL contexts (default 2) at once, and every context is warmed
# when created (one small call per precision: its buffers are sized and its
# graphs captured), so a thread that arrives while the others are pricing does
# not pay that set-up -- whose allocations would wait for the whole device --
# inside its call.

_pool: list = []
_pool_lock = threading.Lock()
_pool_started = False
_tls = threading.local()


def _new_engine() -> _g.Engine:
    eng = _g.Engine(int(os.environ.get("MCD_GPU_DEVICE", "0")))
    for prec in ("fp64", "fp32"):
        eng.monte_carlo_european(100.0, 100.0, 0.05, 0.0, 0.2, 1.0, 0, 4096, 1, precision=prec)
    return eng


class _Lease:
    def __enter__(self) -> _g.Engine:
        global _pool_started
        with _pool_lock:
            if not _pool_started:
                _pool_started = True
                _pool.extend(_new_engine() for _ in range(max(1, int(os.environ.get("MCD_GPU_POOL", "2")))))
            self.eng = _pool.pop() if _pool else None
        if self.eng is None:
            self.eng = _new_engine()
        return self.eng

    def __exit__(self, *exc):
        with _pool_lock:
            _pool.append(self.eng)


def _engine() -> _Lease:
    return _Lease()


def set_precision(precision: str) -> None:
    """"fp64" (default, the reference's arithmetic) or "fp32" for this thread."""
    if precision not in ("fp64", "fp32"):
        raise ValueError("precision must be 'fp64' or 'fp32'")
    _tls.precision = precision


def _prec() -> str:
    return getattr(_tls, "precision", "fp64")


def _opts(options):
    return options if options is not None else McOptions()


# -- closed forms and lattices (module.cpp:179-198) -------------------------------
black_scholes_merton = _g.black_scholes_merton
black76 = _g.black76
kemna_vorst = _g.kemna_vorst
reiner_rubinstein = _g.reiner_rubinstein
lookback_fixed_strike = _g.lookback_fixed_strike
lookback_floating_strike = _g.lookback_floating_strike
digital = _g.digital
forward_price = _g.forward_price
forward_value = _g.forward_value
futures_mark_to_market = _g.futures_mark_to_market
crr_binomial = _g.crr_binomial
crr_binomial_american = _g.crr_binomial_american
heston_semi_analytic = _g.heston_semi_analytic

# -- Monte Carlo pricers (module.cpp:203-233) -------------------------------------


def monte_carlo_european(spot, strike, rate, carry_yield, vol, time, type, path_count, seed, options=None):
    o = _opts(options)
    with _engine() as e:
        return e.monte_carlo_european(spot, strike, rate, carry_yield, vol, time, type, path_count, seed,
                                      antithetic=o.antithetic, precision=_prec())


def monte_carlo_digital(spot, strike, rate, carry_yield, vol, time, type, style, cash_amount, path_count, seed,
                        options=None):
    o = _opts(options)
    with _engine() as e:
        return e.monte_carlo_digital(spot, strike, rate, carry_yield, vol, time, type, style, cash_amount,
                                     path_count, seed, antithetic=o.antithetic, precision=_prec())


def monte_carlo_asian(spot, strike, rate, carry_yield, vol, time, type, strike_style, average_style,
                      monitoring_points, path_count, seed, options=None):
    o = _opts(options)
    with _engine() as e:
        return e.monte_carlo_asian(spot, strike, rate, carry_yield, vol, time, type, strike_style,
                                   average_style, monitoring_points, path_count, seed,
                                   antithetic=o.antithetic, control_variate=o.control_variate,
                                   precision=_prec())


def monte_carlo_barrier(spot, strike, barrier, rate, carry_yield, vol, time, type, direction, knock, rebate,
                        monitoring_points, path_count, seed, options=None):
    o = _opts(options)
    with _engine() as e:
        return e.monte_carlo_barrier(spot, strike, barrier, rate, carry_yield, vol, time, type, direction,
                                     knock, rebate, monitoring_points, path_count, seed,
                                     antithetic=o.antithetic, brownian_bridge=o.brownian_bridge,
                                     precision=_prec())


def monte_carlo_lookback(spot, strike, rate, carry_yield, vol, time, type, style, monitoring_points, path_count,
                         seed, options=None):
    o = _opts(options)
    with _engine() as e:
        return e.monte_carlo_lookback(spot, strike, rate, carry_yield, vol, time, type, style,
                                      monitoring_points, path_count, seed, antithetic=o.antithetic,
                                      precision=_prec())


def monte_carlo_lsm_american(spot, strike, rate, carry_yield, vol, time, type, monitoring_points, path_count,
                             seed):
    with _engine() as e:
        r = e.monte_carlo_lsm_american(spot, strike, rate, carry_yield, vol, time, type, monitoring_points,
                                       path_count, seed, precision=_prec())
    return LsmResult(r.price, r.standard_error)


# -- Greeks (module.cpp:238-256) --------------------------------------------------


def default_bump_sizes(spot, vol, time):
    return _g.lib().mcd_default_bump_sizes(spot, vol, time)


def finite_difference_european(spot, strike, rate, carry_yield, vol, time, type, path_count, seed, bumps):
    with _engine() as e:
        return e.finite_difference_european(spot, strike, rate, carry_yield, vol, time, type, path_count,
                                            seed, bumps, precision=_prec())


def likelihood_ratio_european(spot, strike, rate, carry_yield, vol, time, type, path_count, seed):
    with _engine() as e:
        return LrGreeks(e.likelihood_ratio_european(spot, strike, rate, carry_yield, vol, time, type,
                                                    path_count, seed, precision=_prec()))


def likelihood_ratio_digital(spot, strike, rate, carry_yield, vol, time, type, style, cash_amount, path_count,
                             seed):
    with _engine() as e:
        return LrGreeks(e.likelihood_ratio_digital(spot, strike, rate, carry_yield, vol, time, type, style,
                                                   cash_amount, path_count, seed, precision=_prec()))


def likelihood_ratio_barrier(spot, strike, barrier, rate, carry_yield, vol, time, type, direction, knock, rebate,
                             monitoring_points, path_count, seed):
    with _engine() as e:
        return LrGreeks(e.likelihood_ratio_barrier(spot, strike, barrier, rate, carry_yield, vol, time, type,
                                                   direction, knock, rebate, monitoring_points, path_count,
                                                   seed, precision=_prec()))


def pathwise_european(spot, strike, rate, carry_yield, vol, time, type, path_count, seed):
    with _engine() as e:
        return PathwiseGreeks(e.pathwise_european(spot, strike, rate, carry_yield, vol, time, type,
                                                  path_count, seed, precision=_prec()))


def pathwise_asian(spot, strike, rate, carry_yield, vol, time, type, strike_style, average_style,
                   monitoring_points, path_count, seed):
    with _engine() as e:
        return PathwiseGreeks(e.pathwise_asian(spot, strike, rate, carry_yield, vol, time, type,
                                               strike_style, average_style, monitoring_points, path_count,
                                               seed, precision=_prec()))


# -- Sobol QMC (module.cpp:262-280) -----------------------------------------------


def qmc_sobol_european(spot, strike, rate, carry_yield, vol, time, type, path_count):
    with _engine() as e:
        return QmcResult(e.qmc_sobol_european(spot, strike, rate, carry_yield, vol, time, type, path_count,
                                              precision=_prec()))


def qmc_sobol_asian(spot, strike, rate, carry_yield, vol, time, type, strike_style, monitoring_points,
                    path_count):
    if monitoring_points < 1 or monitoring_points > SOBOL_MAX_DIMENSIONS:
        raise ValueError(f"monitoring_points must be between 1 and {SOBOL_MAX_DIMENSIONS}")
    with _engine() as e:
        return QmcResult(e.qmc_sobol_asian(spot, strike, rate, carry_yield, vol, time, type, strike_style,
                                           monitoring_points, path_count, precision=_prec()))


# -- Heston (module.cpp:282-285) --------------------------------------------------


def heston_qe_european(params, strike, type, monitoring_points, path_count, seed):
    with _engine() as e:
        return e.heston_qe_european(params, strike, type, monitoring_points, path_count, seed,
                                    precision=_prec())


# -- benchmark harness (module.cpp:29-60, 289-292) --------------------------------


def benchmark_european(spot, strike, rate, carry_yield, vol, time, type, path_count, seed, options=None):
    with _engine() as e:
        return e.benchmark_european(spot, strike, rate, carry_yield, vol, time, type, path_count, seed,
                                    options=_opts(options), precision=_prec())
