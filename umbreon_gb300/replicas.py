"""Multi-GPU host logic: frames are independent, so N GPUs run N replicas.

Every rank renders its own frames (the same workload per rank, or its block
of a frame list) with no data exchange; the only collective is the timing
reduction: the job's time is the slowest rank's, its throughput the units of
all ranks over that time.  Works on any torch.distributed backend (NCCL on
GPUs, gloo on the CPU).
"""
from __future__ import annotations

import os
import socket
import subprocess
import sys


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


def barrier() -> None:
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def timed_steps(step, steps: int, sync=lambda: None, device=None) -> dict:
    """The per-rank timed loop of a replica job.

    Every rank runs `steps` calls of ``step()`` between a barrier and a
    ``sync()`` (``torch.cuda.synchronize`` on a GPU) on both sides.  A step
    returns (units, ms): the units it processed and its own duration (CUDA
    events on a GPU).  The job's time is the slowest rank's summed step time,
    its units those of all ranks.  Returns the job figures and this rank's."""
    barrier()
    sync()
    units = ms = 0.0
    for _ in range(steps):
        u, m = step()
        units += u
        ms += m
    sync()
    barrier()
    units_s, ms_max = job_throughput(units, ms, device)
    return {"units_per_s": units_s, "ms_max": ms_max, "units_all": sum_over_ranks(units, device),
            "local_units": units, "local_ms": ms}


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def launch_cmd(n: int, script: str, argv: list[str], port: int | None = None) -> list[str]:
    """torchrun command line that runs `script argv` as n ranks on this node."""
    return [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
            "--master-addr=127.0.0.1", f"--master-port={port or free_port()}", script] + list(argv)


def launch(n: int, script: str, argv: list[str]) -> int:
    """Run `script` as n ranks (one per GPU) when this process was not
    started by torchrun; returns the launcher's exit code."""
    return subprocess.call(launch_cmd(n, script, argv))
