"""Instance sharding across ranks (one process per GPU).

Batched instances are independent, so ranks never exchange data on the solve path: each
rank owns a set of instances (its own synthetic batch for weak scaling, or a cost-balanced
share of one batch for strong scaling, ShardedBatch).  The collectives are the max of the
timings and, for strong scaling, one gather of the shards' results after the solves.
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


def gather_results(shards, local, count, device=None):
    """Whole-batch results from every rank's own shard results (strong scaling).

    shards: the index lists of shard_lpt (the same on every rank); local: (values, grads,
    status) of this rank's shard, in its shard's order.  Returns (values[count],
    grads[count, 5], status[count]) in the batch's order on every rank: one all_gather of a
    padded (max shard, 7) block per rank -- the only exchange, after the solves."""
    import numpy as np
    import torch
    import torch.distributed as dist

    world = len(shards)
    width = max(1, max(len(s) for s in shards))
    v, g, st = local
    block = torch.zeros((width, 7), dtype=torch.float64, device=device)
    n = len(v)
    if n:
        block[:n, 0] = torch.as_tensor(np.asarray(v, dtype=np.float64))
        block[:n, 1:6] = torch.as_tensor(np.asarray(g, dtype=np.float64).reshape(n, 5))
        block[:n, 6] = torch.as_tensor(np.asarray(st, dtype=np.float64))
    if world > 1:
        parts = [torch.empty_like(block) for _ in range(world)]
        dist.all_gather(parts, block)
    else:
        parts = [block]
    values = np.zeros(count)
    grads = np.zeros((count, 5))
    status = np.zeros(count, dtype=np.int32)
    for r, idx in enumerate(shards):
        a = parts[r].cpu().numpy()
        for q, k in enumerate(idx):
            values[k] = a[q, 0]
            grads[k] = a[q, 1:6]
            status[k] = int(a[q, 6])
    return values, grads, status


class ShardedBatch:
    """One batch of problems split over the ranks of the default process group (strong scaling):
    each rank solves its cost-balanced (LPT) shard with its own batch solver on its own GPU, with
    no exchange on the solve path, and results() gathers the whole batch's values, gradients and
    status on every rank.  `make_solver(problems)` builds the rank-local solver (default:
    BatchSolver in the given precision)."""

    def __init__(self, problems, precision: str = "f64", make_solver=None, device=None):
        import torch.distributed as dist

        self.problems = list(problems)
        self.world = dist.get_world_size() if dist.is_available() and dist.is_initialized() else 1
        self.rank = dist.get_rank() if self.world > 1 else 0
        self.shards = shard_lpt(self.problems, self.world)
        self.mine = self.shards[self.rank]
        self.device = device
        if make_solver is None:
            from .batch import BatchSolver

            def make_solver(ps):
                return BatchSolver(ps, precision=precision)
        self.local = make_solver([self.problems[k] for k in self.mine]) if self.mine else None

    def local_cost(self) -> int:
        return sum(cost(self.problems[k]) for k in self.mine)

    def run(self, mode: int = 0, **kw):
        if self.local is not None:
            self.local.run(mode=mode, **kw)

    def results(self):
        import numpy as np

        if self.local is not None:
            local = self.local.results()
        else:
            local = (np.zeros(0), np.zeros((0, 5)), np.zeros(0, dtype=np.int32))
        return gather_results(self.shards, local, len(self.problems), device=self.device)
