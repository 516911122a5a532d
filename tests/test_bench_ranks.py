"""The multi-replica logic of bench.py on CPU: two gloo ranks agree on the slowest rank's
time, the job's throughput counts every rank's work, and the reference arm does its work on
rank 0 only (the other ranks return without output)."""
from __future__ import annotations

import contextlib
import io
import os
import socket
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, queue) -> None:
    import torch.distributed as dist

    sys.path.insert(0, str(ROOT))
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(1.5 + rank, dist, "cpu")
        queue.put((rank, slowest, bench.job_throughput(world, 1e9, 4, slowest)))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_replica():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # every rank sees the slower rank's time; the job did 2 ranks x 4 steps x 1e9 units in it
    assert [r[1] for r in results] == [2.5, 2.5]
    assert all(abs(r[2] - 2 * 4 / 2.5) < 1e-12 for r in results)


def test_single_process_keeps_its_own_time():
    sys.path.insert(0, str(ROOT))
    import bench

    assert bench.max_over_ranks(3.25, None, "cpu") == 3.25
    assert bench.job_throughput(1, 2e9, 5, 2.0) == pytest.approx(5.0)


def test_reference_arm_runs_on_rank_zero_only():
    sys.path.insert(0, str(ROOT))
    import bench

    class Args:
        gpus, steps, warmup = 2, 1, 3

    out = io.StringIO()
    with contextlib.redirect_stdout(out):
        bench.run_reference(Args(), 1)
    assert out.getvalue() == ""
