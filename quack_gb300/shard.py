"""Spreading independent GW systems over the ranks of a one-process-per-GPU job.

The path has no exchange step: a system never spans GPUs, so N GPUs run N independent shares of
a batch (or N replicas of one system) and nothing on the data path talks to another rank.  This
module holds the host-side logic only:

* ``cost``: the dominant work of one system, the Casida eigensolve, ~ nS^3 with nS = o*v;
* ``partition``: greedy longest-processing-time assignment of systems to ranks (largest first,
  each to the currently least loaded rank), deterministic for a given list;
* ``gather``: the per-rank results brought to every rank once the work is done (an all-gather
  of small host arrays; any torch.distributed backend, gloo on CPU).
"""
from __future__ import annotations

import heapq

import numpy as np


def cost(nOrb: int, nO: int, nC: int = 0, nR: int = 0) -> float:
    nS = (nO - nC) * (nOrb - nO - nR)
    return float(nS) ** 3


def partition(costs, world_size: int):
    """Indices of the systems each rank runs (list of lists, ascending within a rank)."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0.0, r) for r in range(world_size)]
    heapq.heapify(heap)
    shares = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + costs[i], r))
    return [sorted(s) for s in shares]


def gather(local_idx, local_values, n_total: int, group=None):
    """Assemble a per-system result array (n_total x ...) on every rank from each rank's
    (indices, values).  Needs an initialised torch.distributed process group."""
    import torch.distributed as dist

    vals = np.asarray(local_values, dtype=np.float64)
    shape_tail = vals.shape[1:]
    payload = [None] * dist.get_world_size(group)
    dist.all_gather_object(payload, (list(map(int, local_idx)), vals.tolist()), group=group)
    out = np.full((n_total,) + shape_tail, np.nan)
    for idx, v in payload:
        if idx:
            out[np.asarray(idx)] = np.asarray(v, dtype=np.float64).reshape((len(idx),) + shape_tail)
    return out
