"""The benchmark's multi-rank host logic on CPU with world_size-2 gloo
process groups: replicas report the slowest rank's step time and the
whole job's units, and the reference arm runs on rank 0 only."""
import os
import socket
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms = 5.0 + 3.0 * rank                      # rank 1 is the slower replica
        t = bench.max_over_ranks(ms, world, device="cpu")
        rate = bench.job_rate(1000, world, t)
        q.put((rank, t, rate))
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slower rank's 8 ms; 2 x 1000 units in 8 ms
    assert [g[1] for g in got] == [8.0, 8.0]
    assert all(abs(g[2] - 2000 / 8e-3) < 1e-6 for g in got)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(4.5, 1) == 4.5
    assert bench.job_rate(826336, 1, 6.5) == pytest.approx(826336 / 6.5e-3)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    sys.path.insert(0, REPO)
    import bench
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("WORLD_SIZE", "2")

    class Args:
        scale, steps, warmup = 64, 1, 0
    # rank 1 returns before building or running anything
    assert bench.reference_arm(Args()) is None
