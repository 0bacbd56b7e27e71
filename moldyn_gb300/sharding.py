"""Replica sharding for multi-GPU ensembles (one process per GPU).

Independent replicas need no per-step exchange, so N GPUs run N disjoint
shares of the ensemble; the only collectives are a barrier and a max over the
ranks' timers around the measured region.  Shares are balanced by estimated
cost with the longest-processing-time rule: replicas sorted by cost
(descending) each go to the currently lightest rank; ties go to the lower
rank, so every rank computes the same assignment independently.
"""
from __future__ import annotations

import heapq

import numpy as np


def replica_cost(n_atoms: np.ndarray, rho: np.ndarray, r_list: float) -> np.ndarray:
    """Pair work per replica: atoms x min(atoms, neighbours inside r_list)."""
    neigh = 4.0 / 3.0 * np.pi * r_list ** 3 * np.asarray(rho, dtype=np.float64)
    return np.asarray(n_atoms, dtype=np.float64) * np.minimum(np.asarray(n_atoms, dtype=np.float64), 1.0 + neigh)


def shard(costs, world: int) -> list:
    """Indices of the replicas each rank owns (LPT on `costs`)."""
    costs = np.asarray(costs, dtype=np.float64)
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world)]
    heapq.heapify(heap)
    out = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(x) for x in out]


def max_over_ranks(value: float, dist=None, device=None) -> float:
    """Max of a per-rank timer across the process group (identity without one)."""
    if dist is None or not dist.is_initialized():
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
