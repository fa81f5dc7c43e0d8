"""Multi-GPU host logic: frames are independent, so N GPUs run N replicas.

Every rank renders its own frames (the same workload per rank, or its block
of a frame list) with no data exchange; the only collective is the timing
reduction: the job's time is the slowest rank's, its throughput the units of
all ranks over that time.  Works on any torch.distributed backend (NCCL on
GPUs, gloo on the CPU).
"""
from __future__ import annotations

import os


def env_ranks():
    """(world_size, rank, local_rank) from the torchrun environment."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def partition(n_items: int, rank: int, world: int) -> range:
    """Contiguous block of items owned by `rank` (sizes differ by at most 1)."""
    base, extra = divmod(n_items, world)
    start = rank * base + min(rank, extra)
    return range(start, start + base + (1 if rank < extra else 0))


def _reduce(value: float, op: str, device=None) -> float:
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(value: float, device=None) -> float:
    return _reduce(value, "max", device)


def sum_over_ranks(value: float, device=None) -> float:
    return _reduce(value, "sum", device)


def job_throughput(local_units: float, local_ms: float, device=None) -> tuple[float, float]:
    """(units of all ranks per second, slowest rank's ms)."""
    ms = max_over_ranks(local_ms, device)
    units = sum_over_ranks(local_units, device)
    return units / (ms / 1e3), ms
