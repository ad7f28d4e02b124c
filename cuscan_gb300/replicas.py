"""Replica bookkeeping for multi-process runs (one process per GPU, torch.distributed).

The fit core is not partitioned across devices: every rank fits its own point set (a replica)
and nothing is exchanged on the data path. The only collective is the timing reduction: the
slowest rank's time defines the aggregate throughput of the job.
"""
from __future__ import annotations

import torch
import torch.distributed as dist


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of rank `rank`'s replica: rank 0 keeps the workload's own seed."""
    return int(base_seed) + 1000 * int(rank)


def slowest(seconds: float, device: str = "cpu") -> float:
    """Maximum of `seconds` over all ranks of the default group (identity without one)."""
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def aggregate_throughput(points_per_rank: int, steps: int, seconds: float,
                         device: str = "cpu") -> tuple[float, float]:
    """(whole-job points per second, slowest rank's seconds) for `steps` fits per rank."""
    world = dist.get_world_size() if (dist.is_available() and dist.is_initialized()) else 1
    worst = slowest(seconds, device)
    return world * points_per_rank * steps / worst, worst
