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
