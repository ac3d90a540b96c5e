"""Voxel sharding and the max-over-ranks timing, with two gloo ranks on CPU."""
import os
import socket

import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from pycompute_gb300.shard import job_throughput, max_over_ranks, shard_range


@pytest.mark.parametrize("n,world", [(0, 1), (10, 3), (8388608, 8), (7, 8), (1025, 2)])
def test_shards_cover_once(n, world):
    covered = []
    sizes = []
    for r in range(world):
        a, b = shard_range(n, r, world)
        covered.extend(range(a, b)) if n < 100000 else None
        sizes.append(b - a)
    assert sum(sizes) == n and max(sizes) - min(sizes) <= 1
    if n < 100000:
        assert covered == list(range(n))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    a, b = shard_range(1000, rank, world)
    times = max_over_ranks([0.5 + rank, 2.0 - rank])
    dist.barrier()
    out[rank] = torch.tensor([a, b, times[0], times[1]], dtype=torch.float64)
    dist.destroy_process_group()


def test_two_rank_max_reduce_gloo():
    world = 2
    out = torch.zeros((world, 4), dtype=torch.float64).share_memory_()
    mp.spawn(_worker, args=(world, _free_port(), out), nprocs=world, join=True)
    assert out[0, 0] == 0 and out[0, 1] == 500 and out[1, 0] == 500 and out[1, 1] == 1000
    assert torch.all(out[:, 2] == 1.5) and torch.all(out[:, 3] == 2.0)
    assert job_throughput([500, 500], 2.0) == 500.0 and job_throughput(500, 2.0, world=2) == 500.0
