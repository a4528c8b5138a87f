"""Assignment of independent grids to ranks for batched runs on several GPUs (one process per GPU).

Grids of a batch share no nodes, so a multi-GPU batch needs no exchange on the data path: each rank
builds a batch from its own grids. This module holds the host-side assignment: size-balanced greedy
packing (largest grid first, onto the rank with the fewest nodes so far; ties to the lower rank), the
same on every rank without communication."""
from __future__ import annotations

import heapq


def assign_by_size(sizes, world):
    """sizes: node count per grid; returns one sorted list of grid indices per rank."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda k: (-int(sizes[k]), k))
    heap = [(0, r) for r in range(world)]
    parts = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        parts[r].append(k)
        heapq.heappush(heap, (load + int(sizes[k]), r))
    return [sorted(p) for p in parts]


def rank_share(sizes, rank, world):
    return assign_by_size(sizes, world)[rank]
