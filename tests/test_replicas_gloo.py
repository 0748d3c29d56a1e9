"""The N > 1 path of bench.py on the CPU: N independent replicas, timed by the
slowest rank (all_reduce MAX), whole-job throughput = N x per-replica work /
that time.  Two gloo ranks stand in for two GPUs (no GPU is touched)."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    t = bench.max_over_ranks(1.0 + 0.5 * rank, world, torch.device("cpu"))
    out[rank] = bench.replica_throughput(world, 823875, 20, t)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_replicas_take_the_slowest_rank(world):
    port = _free_port()
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_rank, args=(world, port, out), nprocs=world, join=True, start_method="spawn")
    slowest = 1.0 + 0.5 * (world - 1)
    expected = world * 823875 * 20 / slowest / 1e9
    assert all(abs(out[r] - expected) <= 1e-12 * expected for r in range(world))
