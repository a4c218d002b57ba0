"""The multi-GPU form of the benchmark is N independent replicas (rays are
independent; the reference splits the screen the same way).  Its host logic,
the max over ranks of the timed region and the whole-job rate, runs here as
two gloo ranks on CPU."""
from __future__ import annotations

import os
import socket

import pytest


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, queue) -> None:
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank), XN_BENCH_BACKEND="gloo")
    import bench
    world_, rank_, _, dist = bench.setup_dist(world)
    assert (world_, rank_) == (world, rank)
    local_ms = 100.0 + 50.0 * rank  # rank 1 is the slow one
    total_ms, value = bench.aggregate_replicas(local_ms, 2_000_000, world, dist)
    queue.put((rank, total_ms, value))
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank_and_sum_the_rays():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    queue = mp.Queue()
    port = _free_port()
    procs = [mp.Process(target=_rank, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    got = sorted(queue.get(timeout=10) for _ in range(2))
    for rank, total_ms, value in got:
        assert total_ms == 150.0
        assert value == pytest.approx(2 * 2_000_000 / (150.0 * 1e3))


def test_one_process_needs_no_process_group():
    import bench
    total_ms, value = bench.aggregate_replicas(40.0, 1_000_000, 1, None)
    assert total_ms == 40.0 and value == pytest.approx(1_000_000 / 40e3)
