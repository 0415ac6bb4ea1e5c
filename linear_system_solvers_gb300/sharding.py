"""Instance sharding across ranks (one process per GPU).

Batched instances are independent, so ranks never exchange data on the solve path: each
rank owns a set of instances (its own synthetic batch for weak scaling, or a cost-balanced
share of one batch for strong scaling) and the only collective is the max of the timings.
"""
from __future__ import annotations


def rank_seed(seed: int, rank: int) -> int:
    """Seed of rank `rank`'s own batch (weak scaling: per-GPU work fixed as N grows)."""
    return seed + rank


def cost(p) -> int:
    return p.nx * p.ny * (p.nt - 1)


def shard_lpt(problems, world: int):
    """Longest-processing-time partition of one batch over `world` ranks (strong scaling):
    returns a list of index lists, one per rank, with near-equal grid-point-step totals."""
    order = sorted(range(len(problems)), key=lambda k: -cost(problems[k]))
    loads = [0] * world
    shards = [[] for _ in range(world)]
    for k in order:
        r = min(range(world), key=lambda q: loads[q])
        shards[r].append(k)
        loads[r] += cost(problems[k])
    return [sorted(s) for s in shards]


def max_over_ranks(values, device=None):
    """Element-wise max of a list of floats over all ranks of the default process group."""
    import torch
    import torch.distributed as dist

    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def sum_over_ranks(values, device=None):
    """Element-wise sum of a list of floats over all ranks of the default process group."""
    import torch
    import torch.distributed as dist

    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return [float(x) for x in t.cpu()]
