"""Multi-GPU layout of independent maps: one process per GPU, whole maps
assigned to ranks, no collective on the data path.

A single map does not shard (a scan's rays cross any spatial split, so a split
map would need a per-scan exchange of ray segments); independent maps do. The
only cross-rank communication is the benchmark's aggregation of throughput and
time (one all_reduce of two numbers after the timed region).
"""
from __future__ import annotations

from typing import Sequence


def assign_maps(sizes: Sequence[int], world_size: int) -> list[int]:
    """Rank of each map: greedy longest-processing-time assignment by scan size
    (points per scan), so that ranks get similar work. Deterministic."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]), i))
    load = [0] * world_size
    rank_of = [0] * len(sizes)
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        rank_of[i] = r
        load[r] += int(sizes[i])
    return rank_of


def my_maps(sizes: Sequence[int], world_size: int, rank: int) -> list[int]:
    return [i for i, r in enumerate(assign_maps(sizes, world_size)) if r == rank]


def aggregate(units: float, seconds: float, group=None):
    """Whole-job throughput: units summed over ranks, time = slowest rank."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return units, seconds
    u = torch.tensor([float(units)], dtype=torch.float64)
    t = torch.tensor([float(seconds)], dtype=torch.float64)
    if dist.get_backend(group) == "nccl":
        u, t = u.cuda(), t.cuda()
    dist.all_reduce(u, op=dist.ReduceOp.SUM, group=group)
    dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return float(u.item()), float(t.item())
