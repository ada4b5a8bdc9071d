"""The multi-GPU path of bench.py is N independent replicas (the SpMV does not
need a collective); its only cross-rank steps are the barrier and the
max-over-ranks timing.  Checked here with two gloo ranks on the CPU."""
from __future__ import annotations

import os
import socket

import pytest

from conftest import ROOT


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out) -> None:
    import sys

    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        slow = bench.replica_max(10.0 + rank, "cpu")
        gbs = bench.replica_throughput(2_000_000_000, 5, world, slow)
        out.put((rank, slow, gbs))
    finally:
        dist.destroy_process_group()


def test_replica_timing_takes_the_slowest_rank():
    import torch.multiprocessing as mp

    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(world))
    for _, slow, gbs in res:
        assert slow == 11.0  # the slower rank's time on every rank
        assert gbs == pytest.approx(2e9 * 5 * world / 11e-3 / 1e9)


def test_single_process_replica_max_is_identity():
    import sys

    sys.path.insert(0, ROOT)
    import bench

    assert bench.replica_max(3.5) == 3.5
