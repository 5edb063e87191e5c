"""One process per GPU, independent work per rank.

The hot path does not shard a single grid: its compact z solves would need a
distributed tridiagonal (or a pencil transpose) and its WENO5 stencil a z halo,
so N GPUs run N independent grids (replicas of the headline tank) or split an
ensemble of independent grids between them.  Neither needs a collective on the
data path; the only communication is host control: a barrier around the timed
region and the maximum of the ranks' times.

The functions take the torch.distributed backend's device ("cuda" with NCCL on
GPU boxes, "cpu" with gloo in the CPU tests), so the same logic is tested on
the host with world size 2.
"""
from __future__ import annotations

import os


def world_from_env() -> tuple[int, int, int]:
    """(world size, rank, local rank) from the torchrun environment."""
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def barrier(world: int) -> None:
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The largest x over the ranks (every rank gets it)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def shard_by_cost(costs, world: int) -> list[list[int]]:
    """Split independent items (grids) between `world` ranks: largest first,
    each to the rank with the least cost so far (LPT; deterministic, ties to
    the lower rank).  Returns the item indices of every rank, each ascending."""
    if world < 1:
        raise ValueError("world size must be at least 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += costs[i]
    return [sorted(p) for p in parts]
