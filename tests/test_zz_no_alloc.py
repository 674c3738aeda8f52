"""The allocation-free batch entry point (mcd_price_batch_static), called
through the C ABI.

It exists for callers that cannot call cudaMalloc (services that reserve all
device memory up front, or code where an allocation's implicit device
synchronisation is not allowed).  Its scratch lives in a fixed __device__ array
instead, so two checks matter: it returns what the allocating entry point
(mcd_price_batch) returns for the same contracts, and it keeps doing so on
consecutive calls that reuse that array.  Results must agree within the 1e-12
relative price tolerance the parity tests use (they are in fact bitwise equal:
same kernels, same slab tree).

This file sorts last so that a run stopping at the first failure has already
run every other test; it also passes alone in a fresh process.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

PRICE_REL = 1e-12


def _static_fn(gpu_lib):
    f = gpu_lib.lib().mcd_price_batch_static
    f.restype = C.c_int
    f.argtypes = [C.c_void_p, C.c_size_t, C.c_int, C.c_void_p, C.c_void_p, C.c_char_p, C.c_size_t]
    return f


def _batch(gpu_lib, n, seed):
    rng = np.random.default_rng(seed)
    c = gpu_lib.contracts(n)
    c["product"] = rng.integers(0, 5, n)
    c["type"] = rng.integers(0, 2, n)
    c["spot"] = 100.0
    c["strike"] = rng.uniform(80, 120, n)
    c["rate"] = rng.uniform(0, .06, n)
    c["vol"] = rng.uniform(.1, .5, n)
    c["time"] = rng.uniform(.25, 2, n)
    c["monitoring_points"] = rng.integers(1, 60, n)
    c["path_count"] = rng.integers(0, 30000, n)
    c["seed"] = 42 + np.arange(n)
    c["direction"] = rng.integers(0, 2, n)
    c["knock"] = rng.integers(0, 2, n)
    c["barrier"] = np.where(c["direction"] == 0, 100 * (1 + rng.uniform(.05, .3, n)),
                            100 * (1 - rng.uniform(.05, .3, n)))
    c["strike_style"] = rng.integers(0, 2, n)
    c["average_style"] = rng.integers(0, 2, n)
    c["antithetic"] = rng.integers(0, 2, n)
    c["brownian_bridge"] = rng.integers(0, 2, n)
    c["control_variate"] = rng.integers(0, 2, n)
    return c


def _call_static(fn, gpu_lib, c, precision):
    out = np.zeros(len(c), dtype=gpu_lib.RESULT_DTYPE)
    msg = C.create_string_buffer(256)
    rc = fn(c.ctypes.data, len(c), precision, out.ctypes.data, None, msg, len(msg))
    assert rc == 0, msg.value.decode()
    return out


@pytest.mark.parametrize("precision", [0, 1])
def test_static_matches_allocating_entry_on_consecutive_calls(gpu_lib, precision):
    fn = _static_fn(gpu_lib)
    first = _batch(gpu_lib, 80, seed=5)
    second = _batch(gpu_lib, 48, seed=6)   # smaller: stale slots of the first call must not leak
    with gpu_lib.Engine(0) as eng:
        want1 = eng.price_batch(first, precision)
        want2 = eng.price_batch(second, precision)
    got1 = _call_static(fn, gpu_lib, first, precision)
    got2 = _call_static(fn, gpu_lib, second, precision)
    for got, want in ((got1, want1), (got2, want2)):
        assert (got["path_count"] == want["path_count"]).all()
        assert np.all(np.abs(got["price"] - want["price"]) <= PRICE_REL * np.abs(want["price"]))
        assert np.all(np.abs(got["standard_error"] - want["standard_error"])
                      <= PRICE_REL * np.abs(want["standard_error"]))
        assert got.tobytes() == want.tobytes()


def test_static_rejects_sizes_beyond_its_limit(gpu_lib):
    fn = _static_fn(gpu_lib)
    too_many = gpu_lib.contracts(4097)
    out = np.zeros(4097, dtype=gpu_lib.RESULT_DTYPE)
    msg = C.create_string_buffer(256)
    rc = fn(too_many.ctypes.data, 4097, 1, out.ctypes.data, None, msg, len(msg))
    assert rc == -1
    assert b"4096" in msg.value
    big = gpu_lib.contracts(2)
    big["product"] = 0
    big["spot"] = big["strike"] = 100.0
    big["vol"] = .2
    big["time"] = 1.0
    big["path_count"] = 200000 * 4096  # 200000 slabs each: over the 262144-slab limit together
    rc = fn(big.ctypes.data, 2, 1, out.ctypes.data, None, msg, len(msg))
    assert rc == -1 and b"262144" in msg.value
    # still usable afterwards
    ok = _batch(gpu_lib, 4, seed=9)
    _call_static(fn, gpu_lib, ok, 1)


def test_static_matches_oracle_directly(gpu_lib, orc):
    """The allocation-free entry point against the CPU oracle (the reference's
    algorithm restated), without going through the allocating entry point:
    FP64 prices within 1e-12 relative on identical draws."""
    import oracle as O
    fn = _static_fn(gpu_lib)
    c = _batch(gpu_lib, 24, seed=12)
    c["path_count"] = np.maximum(c["path_count"], 1)
    for _ in range(2):  # two calls in a row on the shared array
        got = _call_static(fn, gpu_lib, c, 0)
        arr = (O.Contract * len(c))()
        for i, row in enumerate(c):
            for name in row.dtype.names:
                setattr(arr[i], name, row[name].item())
        want = (O.McResult * len(c))()
        orc.orc_price_batch(arr, len(c), 1, 0, want)
        for i in range(len(c)):
            assert got["path_count"][i] == want[i].path_count
            assert abs(got["price"][i] - want[i].price) <= PRICE_REL * abs(want[i].price) + 1e-300, (i, c[i])


def test_static_rejects_path_counts_whose_slab_count_overflows(gpu_lib):
    """2^44 paths and more need 2^32 slabs or more: rejected, never wrapped."""
    fn = _static_fn(gpu_lib)
    out = np.zeros(1, dtype=gpu_lib.RESULT_DTYPE)
    msg = C.create_string_buffer(256)
    for paths in (1 << 44, (1 << 44) + 1, 1 << 53):
        c = gpu_lib.contracts(1)
        c["product"] = 0
        c["spot"] = c["strike"] = 100.0
        c["vol"] = .2
        c["time"] = 1.0
        c["path_count"] = paths
        rc = fn(c.ctypes.data, 1, 1, out.ctypes.data, None, msg, len(msg))
        assert rc == -1, (paths, msg.value)
        assert msg.value


def test_static_setup_call_with_no_contracts(gpu_lib):
    fn = _static_fn(gpu_lib)
    msg = C.create_string_buffer(256)
    assert fn(None, 0, 1, None, None, msg, len(msg)) == 0, msg.value
