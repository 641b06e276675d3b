"""The multi-GPU contract of bench.py on CPU: N replicas (one per rank, no data exchange) report the whole
job's rate, every rank's work over the slowest rank's time, from one max all-reduce; world-size-2 `gloo`
ranks stand in for the GPUs. Under torchrun the reference arm runs on rank 0 only."""
import os
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    import sys

    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r took r + 1 seconds for 100 units; the job did 100 * world units in the slowest time
        out[rank] = bench.replica_rate(world, 100, rank + 1.0)
        dist.barrier()
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2, 3])
def test_replica_rate_takes_the_slowest_rank(world):
    ctx = mp.get_context("spawn")
    out = ctx.Manager().dict()
    mp.start_processes(rank_main, args=(world, free_port(), out), nprocs=world, join=True, start_method="spawn")
    assert sorted(out.keys()) == list(range(world))
    for r in range(world):
        assert out[r] == pytest.approx(world * 100 / world)  # slowest rank: world seconds


def test_single_rank_rate():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(1, 8192, 0.5) == pytest.approx(16384.0)


def test_reference_arm_other_ranks_exit(monkeypatch):
    import sys
    sys.path.insert(0, ROOT)
    import bench
    monkeypatch.setenv("RANK", "1")

    class Args:
        steps, warmup, ref_points, gpus = 1, 0, 8, 2
    assert bench.run_reference(Args()) == 0
