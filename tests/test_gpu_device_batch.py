"""mcd_price_batch_device: device-resident contracts and results, through the C ABI.

* The device-resident call returns bitwise what mcd_price_batch returns.
* Contracts rewritten in place on the caller's stream (same pointer, same
  count) are priced as rewritten: the launch plan is keyed on a digest of the
  records, computed on that stream, not only on the pointer.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _batch(M, n, seed):
    rng = np.random.default_rng(seed)
    c = M.contracts(n)
    c["product"] = rng.integers(0, 5, n)
    c["type"] = rng.integers(0, 2, n)
    c["spot"] = 100.0
    c["strike"] = rng.uniform(80, 120, n)
    c["rate"] = rng.uniform(0, .06, n)
    c["vol"] = rng.uniform(.1, .5, n)
    c["time"] = rng.uniform(.25, 2, n)
    c["monitoring_points"] = rng.integers(1, 60, n)
    c["path_count"] = rng.integers(1, 30000, n)
    c["seed"] = 42 + np.arange(n)
    c["direction"] = rng.integers(0, 2, n)
    c["knock"] = rng.integers(0, 2, n)
    c["barrier"] = np.where(c["direction"] == 0, 100 * (1 + rng.uniform(.05, .3, n)),
                            100 * (1 - rng.uniform(.05, .3, n)))
    c["strike_style"] = rng.integers(0, 2, n)
    c["average_style"] = rng.integers(0, 2, n)
    return c


def test_device_batch_equals_host_batch_and_follows_in_place_rewrites(engine, gpu_lib):
    torch = pytest.importorskip("torch")
    M = gpu_lib
    n = 64
    first, second = _batch(M, n, 1), _batch(M, n, 2)
    side = torch.cuda.Stream()
    d_c = torch.from_numpy(first.view(np.uint8).copy()).cuda()
    d_r = torch.zeros(n * M.RESULT_DTYPE.itemsize, dtype=torch.uint8, device="cuda")

    def device_call(prec):
        engine.price_batch_device(d_c.data_ptr(), n, d_r.data_ptr(), prec, side.cuda_stream)
        side.synchronize()
        return np.frombuffer(d_r.cpu().numpy().tobytes(), dtype=M.RESULT_DTYPE)

    # Host results first: a host-array call re-uploads the context's plan
    # buffers, so it must not sit between the device calls checked below.
    want = {(k, p): engine.price_batch(c, p).tobytes()
            for k, c in (("first", first), ("second", second)) for p in ("fp32", "fp64")}
    torch.cuda.synchronize()
    for prec in ("fp32", "fp64"):
        assert device_call(prec).tobytes() == want[("first", prec)]
    # Same pointer, count and precision; new content written on the caller's stream.
    with torch.cuda.stream(side):
        d_c.copy_(torch.from_numpy(second.view(np.uint8).copy()).to("cuda"))
    assert device_call("fp64").tobytes() == want[("second", "fp64")]
    assert device_call("fp64").tobytes() == want[("second", "fp64")]  # the new plan is reused
    # And back again: the plan of the first content is rebuilt, not assumed.
    with torch.cuda.stream(side):
        d_c.copy_(torch.from_numpy(first.view(np.uint8).copy()).to("cuda"))
    assert device_call("fp64").tobytes() == want[("first", "fp64")]
