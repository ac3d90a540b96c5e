"""Voxel sharding across ranks (one process per GPU).

Voxels are independent, so a job over N voxels splits into contiguous
shards with no data exchange; the only collectives are the timing barrier and
a max-reduce of per-rank times (the job is as slow as its slowest rank).
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def shard_range(n_total: int, rank: int, world: int) -> tuple[int, int]:
    """[start, stop) of rank's contiguous shard; shard sizes differ by at most one."""
    if world < 1 or not 0 <= rank < world or n_total < 0:
        raise ValueError("bad shard request")
    base, extra = divmod(n_total, world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def max_over_ranks(values: list[float], device=None) -> list[float]:
    """Element-wise maximum of per-rank values (identity without a process group)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return list(values)
    t = torch.tensor(values, dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return t.tolist()


def job_throughput(units_per_rank: list[int] | int, seconds_max: float, world: int = 1) -> float:
    """Whole-job units per second: all ranks' units over the slowest rank's time."""
    total = sum(units_per_rank) if isinstance(units_per_rank, list) else units_per_rank * world
    return total / seconds_max
