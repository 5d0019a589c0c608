"""Replica runs: one process per GPU, each stepping its own copy of the workload.

The time step does not shard (the pressure solve couples every cell of the box),
so N GPUs run N independent replicas and exchange nothing on the data path.  The
only cross-rank traffic is the timing: each rank's device time is reduced with a
MAX, and the whole-job throughput counts the cells of every replica over that
slowest time.  Works over any torch.distributed backend (nccl on GPUs, gloo on
host cores); without an initialised process group it is the single-process case.
"""
from __future__ import annotations

import os


def world() -> tuple[int, int]:
    """(rank, world size) from the launcher's environment."""
    return int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))


def _dist():
    import torch.distributed as dist
    return dist if dist.is_available() and dist.is_initialized() else None


def barrier() -> None:
    d = _dist()
    if d is not None:
        d.barrier()


def max_over_ranks(x: float) -> float:
    """The largest value of `x` over all ranks (the slowest replica's time)."""
    d = _dist()
    if d is None or d.get_world_size() == 1:
        return float(x)
    import torch
    dev = "cuda" if d.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    d.all_reduce(t, op=d.ReduceOp.MAX)
    return float(t.item())


def throughput(cells_per_replica: int, steps: int, seconds: float) -> float:
    """Whole-job cell-updates/s: every replica's cells over the slowest replica's
    time (the time must already be the maximum over ranks)."""
    d = _dist()
    n = d.get_world_size() if d is not None else 1
    if seconds <= 0:
        raise ValueError("non-positive timed region")
    return n * cells_per_replica * steps / seconds
