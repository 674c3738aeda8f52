"""The multi-GPU form of the path (replicas: each rank prices its own book, no
collective on the data) exercised on CPU with two gloo ranks: distinct pricing seeds
per rank with identical contract terms, and the job time as the slowest rank's."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, root, out):
    import sys
    sys.path[:0] = [root, os.path.join(root, "derivative-pricing_gb300")]
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import bench
        c = bench.make_batch(64, rank=rank)
        seeds = [None] * world
        terms = [None] * world
        dist.all_gather_object(seeds, c["seed"].tolist())
        dist.all_gather_object(terms, c[["strike", "vol", "time", "monitoring_points", "path_count"]].tolist())
        slowest = bench.max_over_ranks(10.0 + rank)
        if rank == 0:
            out.put((seeds, terms, slowest))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replicas():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, root, q)) for r in range(2)]
    for p in procs:
        p.start()
    seeds, terms, slowest = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert not set(seeds[0]) & set(seeds[1])          # each replica its own paths
    assert seeds[0][0] == 42 and seeds[1][0] == 42 + 64
    assert terms[0] == terms[1]                       # the same book terms
    assert slowest == 11.0                            # max over ranks


def test_single_process_max_is_identity():
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert np.array_equal(bench.make_batch(8)["seed"], 42 + np.arange(8))
