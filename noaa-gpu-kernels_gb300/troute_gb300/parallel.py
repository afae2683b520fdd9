"""Sharding of batched routing across ranks (one process per GPU).

Independent basins and ensemble members need no exchange between GPUs: each
rank routes its share in one persistent launch and the results are gathered.
A single river tree does not shard without a per-step exchange of the
outflows across cut edges, so it runs as replicas (one copy per rank).
"""
from __future__ import annotations

import heapq


def partition(sizes, world_size: int):
    """Greedy longest-processing-time bin packing of networks (by segment
    count, the work per step) onto `world_size` ranks. Returns one sorted list
    of network indices per rank; every index appears exactly once."""
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-sizes[i], i))
    heap = [(0, r) for r in range(world_size)]
    heapq.heapify(heap)
    parts = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + sizes[i], r))
    return [sorted(p) for p in parts]


def member_range(n_members: int, world_size: int, rank: int):
    """Contiguous ensemble members of `rank` (balanced to within one)."""
    base, extra = divmod(n_members, world_size)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)
