"""Multi-rank logic on CPU (gloo, world_size 2): instance sharding, the max-over-ranks timing
reduction and the sum of the ranks' work used by bench.py under torchrun."""
import os
import socket

import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from linear_system_solvers_gb300.batch import draw_batch
    from linear_system_solvers_gb300.sharding import max_over_ranks, rank_seed, shard_lpt, sum_over_ranks

    mine = draw_batch(8, seed=rank_seed(20261203, rank))
    times = max_over_ranks([1.0 + rank, 10.0 - rank])
    work = sum_over_ranks([float(100 + rank)])
    shards = shard_lpt(draw_batch(64), world)
    out.put((rank, mine[0].kappa, times + work, shards[rank]))
    dist.destroy_process_group()


def test_two_rank_gloo_sharding_and_max():
    import multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, k0, t0, s0), (r1, k1, t1, s1) = res
    assert k0 != k1                      # own batch per rank (weak scaling)
    assert t0 == t1 == [2.0, 10.0, 201.0]  # max over ranks of each timing; sum of the work
    assert not set(s0) & set(s1) and len(s0) + len(s1) == 64


def test_lpt_shards_balance_cost():
    from linear_system_solvers_gb300.batch import draw_batch
    from linear_system_solvers_gb300.sharding import cost, shard_lpt

    probs = draw_batch(512)
    for world in (2, 4, 8):
        shards = shard_lpt(probs, world)
        loads = [sum(cost(probs[k]) for k in s) for s in shards]
        assert max(loads) / min(loads) < 1.02
        assert sorted(k for s in shards for k in s) == list(range(512))


class _OracleBatch:
    """CPU stand-in for the rank-local batch solver (test only): values V(eval_s, eval_v) from the
    oracle's surfaces; gradients a deterministic function of the instance so the gather of every
    column is checked."""

    def __init__(self, problems):
        self.problems = problems
        self.out = None

    def run(self, mode=0, **kw):
        import numpy as np

        from oracle import oracle as O

        vals, grads, status = [], [], []
        for p in self.problems:
            op = O.Problem(**p.pde_fields())
            surf = O.solve(op, "f64")
            x, y = O.grid(op, "f64")
            i = int(np.searchsorted(x, p.eval_s)) - 1
            j = int(np.searchsorted(y, p.eval_v)) - 1
            vals.append(float(surf[i, j]))
            grads.append([p.kappa, p.theta_v, p.sigma, p.rho, p.rate * mode])
            status.append(int(not np.all(np.isfinite(surf))))
        self.out = (np.array(vals), np.array(grads), np.array(status, dtype=np.int32))

    def results(self):
        return self.out


def _small_batch():
    from linear_system_solvers_gb300.batch import draw_batch

    probs = draw_batch(12, seed=99)
    for k, p in enumerate(probs):
        p.nx, p.ny, p.nt = 16 + 4 * (k % 5), 10 + 2 * (k % 3), 6 + k
    return probs


def _strong_worker(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from linear_system_solvers_gb300.sharding import ShardedBatch

    sb = ShardedBatch(_small_batch(), make_solver=_OracleBatch)
    sb.run(mode=1)
    v, g, s = sb.results()
    out.put((rank, sb.mine, sb.local_cost(), v.tolist(), g.tolist(), s.tolist()))
    dist.destroy_process_group()


def test_two_rank_strong_scaling_gathers_the_single_rank_results():
    """One batch split over two gloo ranks by cost: each rank solves only its shard, and the
    gathered values, gradients and status equal those of one rank solving the whole batch."""
    import multiprocessing as mp

    import numpy as np

    from linear_system_solvers_gb300.sharding import ShardedBatch

    single = ShardedBatch(_small_batch(), make_solver=_OracleBatch)  # no process group: one rank
    single.run(mode=1)
    v1, g1, s1 = single.results()
    assert single.world == 1 and single.mine == list(range(12))

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_strong_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=180) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, m0, c0, v0, ga, sa), (r1, m1, c1, vb, gb, sb) = res
    assert not set(m0) & set(m1) and sorted(m0 + m1) == list(range(12))
    assert max(c0, c1) / min(c0, c1) < 1.5
    for v, g, s in ((v0, ga, sa), (vb, gb, sb)):
        assert np.array_equal(np.array(v), v1)
        assert np.array_equal(np.array(g), g1)
        assert np.array_equal(np.array(s), s1)
