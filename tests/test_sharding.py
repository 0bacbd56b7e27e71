"""Multi-rank host logic on CPU: replica sharding and the max-over-ranks
timer, run as two gloo ranks (world_size 2) on 127.0.0.1."""
from __future__ import annotations

import os
import socket

import numpy as np
import pytest


def test_lpt_shard_covers_and_balances():
    from moldyn_gb300.sharding import replica_cost, shard
    rng = np.random.default_rng(0)
    n = np.rint(np.exp(rng.uniform(np.log(4), np.log(40), 512))).astype(int) ** 3
    rho = rng.uniform(0.01, 0.9, 512)
    c = replica_cost(n, rho, 2.8)
    for world in (1, 2, 4, 8):
        parts = shard(c, world)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(512))
        loads = [c[p].sum() for p in parts]
        assert max(loads) <= 1.05 * (c.sum() / world) + c.max()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from moldyn_gb300.sharding import max_over_ranks, shard
    costs = np.arange(1, 21, dtype=float)
    mine = shard(costs, world)[rank]
    import torch
    sizes = [torch.zeros(1) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([float(len(mine))]))
    t = max_over_ranks(1.0 + rank, dist)
    dist.barrier()
    out[rank] = (mine, [int(s.item()) for s in sizes], t)
    dist.destroy_process_group()


def test_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    world = 2
    port = _free_port()
    with mp.get_context("spawn").Manager() as m:
        out = m.dict()
        mp.spawn(_worker, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    parts = [res[r][0] for r in range(world)]
    assert sorted(parts[0] + parts[1]) == list(range(20))
    assert res[0][1] == [len(parts[0]), len(parts[1])]
    assert res[0][2] == res[1][2] == 2.0
