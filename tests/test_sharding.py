"""Sharding of batched problems over ranks: every rank computes the same
partition without communicating; checked with two gloo ranks on the CPU."""
import os
import socket

import pytest

from am_ml_suite_gb300.sharding import partition, problem_cost


def test_partition_covers_every_problem_once_and_balances():
    costs = [problem_cost((32 + 7 * i % 65, 16 + 5 * i % 33, 8 + 3 * i % 41)) for i in range(256)]
    for world in (1, 2, 3, 8):
        parts = partition(costs, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(256))
        loads = [sum(costs[i] for i in p) for p in parts]
        assert max(loads) - min(loads) <= max(costs)  # LPT bound
    with pytest.raises(ValueError):
        partition(costs, 0)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, costs, q):
    import torch
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = partition(costs, world)[rank]
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    # the whole-job count and the max-over-ranks time, as the batched bench reduces them
    t = torch.tensor([float(rank + 1), float(len(mine))], dtype=torch.float64)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    q.put((rank, gathered, float(tmax[0]), int(t[1])))
    dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_disjoint_shares():
    import multiprocessing as mp

    costs = [problem_cost((32 + i % 60, 16 + i % 30, 8 + i % 40)) for i in range(40)]
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, costs, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, gathered, tmax, total in out:
        assert gathered[0] == partition(costs, 2)[0] and gathered[1] == partition(costs, 2)[1]
        assert not set(gathered[0]) & set(gathered[1])
        assert tmax == 2.0 and total == 40
