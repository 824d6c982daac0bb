"""Replica execution over several GPUs of one node.

The simulate path does not shard: a register of up to 30 qubits (8 GiB c64)
fits one GPU, so N GPUs run N independent registers (or N slices of a stream
of independent circuits) with no data-path collective.  What is shared is
host-side bookkeeping, kept here so that it is tested on CPU with `gloo`
ranks:

* `rank_seed`    — the seed each rank draws its synthetic input from;
* `partition`    — independent circuits split over ranks by cost
                   (longest-processing-time first), so each rank's slice of a
                   sweep takes about the same device time;
* `reduce_timing` — the whole-job figure: the slowest rank's time and the sum
                   of the units all ranks processed.
"""
from __future__ import annotations

from typing import Sequence


def rank_seed(base: int, rank: int) -> int:
    return int(base) + int(rank)


def partition(costs: Sequence[float], world: int) -> list[list[int]]:
    """Indices of `costs` split into `world` lists: items in decreasing cost
    (ties by index) each go to the rank with the least load so far (ties by
    rank).  Deterministic, so every rank computes the same split."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(costs[i])
    for p in parts:
        p.sort()
    return parts


def reduce_timing(ms: float, units: float, device=None) -> tuple[float, float]:
    """(max over ranks of ms, sum over ranks of units).  Without an
    initialised process group (one rank) the inputs come back unchanged.
    `device` is where the reduction tensor lives (a CUDA device for NCCL,
    None for gloo)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(ms), float(units)
    t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(u, op=dist.ReduceOp.SUM)
    return float(t.item()), float(u.item())
