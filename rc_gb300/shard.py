"""Replica / shard bookkeeping for one process per GPU.

The gridding path shards by independent units (channels, facets, data sets
each own a grid; the reference distributes exactly these as DNA actors,
MS6/programs/continuum.hs:134-141).  Units are assigned to ranks by cost
(longest first onto the least-loaded rank); ranks exchange nothing on the data
path; the only collective is the max of the step time for reporting.
"""
from __future__ import annotations

import heapq


def partition(costs, world):
    """Greedy longest-processing-time assignment: list of unit indices per rank."""
    heap = [(0.0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for u in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        load, r = heapq.heappop(heap)
        out[r].append(u)
        heapq.heappush(heap, (load + float(costs[u]), r))
    return [sorted(x) for x in out]


def my_units(costs, world, rank):
    return partition(costs, world)[rank]


def max_over_ranks(value, device=None):
    """Max of a float over the process group (identity without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
