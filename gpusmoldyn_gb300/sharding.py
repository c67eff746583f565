"""Assignment of independent ensemble instances to ranks (one GPU each).

Instances never interact, so a multi-GPU ensemble is a partition of the
instance list: no collective touches particle data.  The partition balances
particles per rank with the longest-processing-time greedy rule (largest
instance first, to the least-loaded rank), which is deterministic, so every
rank computes the same assignment without communicating.
"""
from __future__ import annotations

import heapq


def balance(counts, world):
    """Return `world` lists of instance indices with near-equal particle sums."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(counts)), key=lambda k: (-int(counts[k]), k))
    heap = [(0, r) for r in range(world)]
    out = [[] for _ in range(world)]
    for k in order:
        load, r = heapq.heappop(heap)
        out[r].append(k)
        heapq.heappush(heap, (load + int(counts[k]), r))
    return [sorted(v) for v in out]


def my_instances(counts, world, rank):
    return balance(counts, world)[rank]
