"""The multi-rank plumbing of bench.py on CPU: two gloo ranks (the GPU run
uses NCCL the same way).  Each rank runs its own replica, so the only
cross-rank steps are the barrier and the max over ranks of every timed
figure; the reference arm runs on rank 0 alone."""
import os
import socket
import sys

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, ws, port, out):
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        barrier, max_over_ranks = bench.rank_ops(dist, "cpu")
        barrier()
        t = max_over_ranks(0.5 + rank)          # per-rank times 0.5 and 1.5 s
        out[rank] = t
        barrier()
    finally:
        dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ws, port = 2, _free_port()
    out = torch.zeros(ws, dtype=torch.float64).share_memory_()
    mp.spawn(_rank_main, args=(ws, port, out), nprocs=ws, join=True)
    assert out.tolist() == [1.5, 1.5]           # every rank reports the slowest


def test_single_rank_ops_are_identity():
    import bench
    barrier, max_over_ranks = bench.rank_ops(None, "cpu")
    barrier()
    assert max_over_ranks(0.25) == 0.25


def test_aggregate_is_whole_job():
    import bench
    # 2 replicas of 4,194,304 cells, 100 steps in 0.1 s
    assert bench.aggregate_mlups(2, 4194304, 100, 0.1) == pytest.approx(8388.608)
    assert bench.aggregate_mlups(1, 4194304, 100, 0.1) == pytest.approx(4194.304)


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")

    class A:
        steps, warmup = 1, 0
    assert bench.run_reference(A()) == 0      # returns at once, no oracle work


def test_both_arms_print_the_same_config():
    """The reference arm and this arm build their config from one function,
    so the two JSON lines name the same workload at every world size."""
    import inspect

    import bench
    for ws in (1, 2, 8):
        assert bench.bench_config(ws) == bench.bench_config(ws)
    for arm in (bench.run_reference, bench.run_ours):
        assert '"config": bench_config(ws)' in inspect.getsource(arm), arm.__name__
