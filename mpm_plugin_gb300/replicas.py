"""Several GPUs as independent replicas: the only multi-GPU form of this path.

A single scene has no data exchange to shard over (the reference is one process on one GPU,
mpm_core/backends/warp/solver.py:32), so each rank runs its own scenes and nothing crosses ranks during a
step. Ranks meet only around a measurement: a barrier before and after, the slowest rank's time and the
sum of the units all ranks processed (reduce_timing). A set of independent scenes is split over the ranks
by estimated cost (shard), largest first onto the least-loaded rank, the same split on every rank.
"""

from __future__ import annotations

import os


def dist_env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the launcher's environment (torchrun), (1, 0, 0) without it."""
    return (int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(costs, rank: int, world: int) -> list[int]:
    """Indices of the items this rank takes: greedy largest-cost-first onto the least-loaded rank (ties to
    the lower rank), so every rank computes the same assignment; returned in ascending order."""
    load = [0.0] * world
    owner = {}
    for i in sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i)):
        r = min(range(world), key=lambda r: (load[r], r))
        owner[i] = r
        load[r] += float(costs[i])
    return [i for i in range(len(costs)) if owner[i] == rank]


def reduce_timing(seconds: float, units: float, device=None) -> tuple[float, float]:
    """(slowest rank's seconds, units summed over ranks); the values themselves on one rank."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(seconds), float(units)
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())


def aggregate_rate(seconds: float, units: float, device=None) -> float:
    """Whole-job throughput: all ranks' units over the slowest rank's time."""
    t, u = reduce_timing(seconds, units, device)
    return u / t if t > 0 else 0.0
