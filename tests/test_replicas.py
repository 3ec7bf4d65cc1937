"""The multi-GPU path of bench.py runs replicas (one process per GPU, the
units sharded by rank, no collective in the data path).  On CPU: two gloo
ranks reduce their timings exactly as the bench does over NCCL (slowest rank's
time, summed work), and the reference arm runs on rank 0 only."""
import os
import socket

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, queue):
    import sys

    import torch.distributed as dist
    sys.path.insert(0, REPO)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    ms, cells = bench.reduce_over_ranks(10.0 + 5.0 * rank, 1000 * (rank + 1), "cpu")
    dist.barrier()
    queue.put((rank, ms, cells))
    dist.destroy_process_group()


def test_reduce_over_ranks_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    queue = ctx.SimpleQueue()
    mp.start_processes(_rank, args=(2, _free_port(), queue), nprocs=2, join=True, start_method="spawn")
    got = sorted(queue.get() for _ in range(2))
    # every rank sees the job's time (the slowest rank) and the summed work
    assert got == [(0, 15.0, 3000.0), (1, 15.0, 3000.0)]


def test_reference_arm_runs_on_rank_zero_only(monkeypatch):
    import bench
    monkeypatch.setenv("WORLD_SIZE", "2")
    monkeypatch.setenv("RANK", "1")
    monkeypatch.setenv("LOCAL_RANK", "1")
    assert bench.run_reference(None) == 0   # no work, no output, exit status 0


@pytest.mark.parametrize("env,expect", [({}, (1, 0, 0)), ({"WORLD_SIZE": "4", "RANK": "3", "LOCAL_RANK": "3"}, (4, 3, 3))])
def test_dist_env(monkeypatch, env, expect):
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        monkeypatch.delenv(k, raising=False)
    for k, v in env.items():
        monkeypatch.setenv(k, v)
    assert bench.dist_env() == expect
