"""The N > 1 path on CPU: two gloo ranks run bench.py's aggregation (replicas only).

Pairs are independent, so ranks never exchange data; the only collective is the
max over ranks of the step time, and the whole-job value is every rank's cells
over the slowest time.
"""
from __future__ import annotations

import os
import socket

import pytest
import torch.multiprocessing as mp

from conftest import REPO


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank: int, world: int, port: int, q):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms = bench.max_over_ranks(5.0 + 3.0 * rank, world)       # rank 1 is the slower one
    value = bench.replica_throughput(1_000_000_000, ms, world)
    dist.barrier()
    q.put((rank, ms, value))
    dist.destroy_process_group()


def test_two_gloo_ranks_take_the_max_time_and_sum_the_cells():
    world, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=5) for _ in range(world))
    for rank, ms, value in got:
        assert ms == pytest.approx(8.0)                    # the max over ranks
        assert value == pytest.approx(2 * 1e9 / 8e-3 / 1e9)  # both replicas' cells / slowest time


def test_single_rank_needs_no_process_group():
    import sys
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_throughput(2_000_000_000, 4.0, 1) == pytest.approx(500.0)
