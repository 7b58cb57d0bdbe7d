"""Placement of independent work on the ranks of a multi-GPU run.

A single triangular solve does not shard along its rows (every level
depends on all the levels before it), so one system with one right-hand
side runs as a replica per GPU.  Its right-hand-side columns do shard: each
rank can solve a block of them against its own copy of the factor
(column_range).  A batch of
independent systems does: each rank takes a subset and solves it with its
own batched plan, and no data crosses ranks (no collective on the data
path).  Systems are placed by longest-processing-time-first greedy bin
packing on their cost (stored entries plus rows, the executor's work), so
the slowest rank's load is within 4/3 of optimal.
"""
from __future__ import annotations

import heapq
from typing import List, Sequence


def system_cost(n: int, nnz: int) -> int:
    return int(n) + int(nnz)


def partition_systems(costs: Sequence[int], world: int) -> List[List[int]]:
    """Indices of the systems each rank solves, each list in ascending order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    heap = [(0, r) for r in range(world)]
    heapq.heapify(heap)
    out: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + int(costs[i]), r))
    return [sorted(v) for v in out]


def rank_systems(costs: Sequence[int], rank: int, world: int) -> List[int]:
    return partition_systems(costs, world)[rank]


def column_range(k: int, rank: int, world: int):
    """The contiguous block of right-hand-side columns [start, stop) a rank
    solves when the k columns of one solve are split over the ranks: every
    rank reads the whole factor, the columns are independent, and the sizes
    differ by at most one."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("need 0 <= rank < world")
    base, extra = divmod(int(k), world)
    start = rank * base + min(rank, extra)
    return start, start + base + (1 if rank < extra else 0)


def shard_systems(systems: Sequence, rank: int, world: int):
    """The rank's share of a batch of (n, p, i, x) systems: (indices,
    systems), placed by partition_systems on each system's rows plus stored
    entries."""
    costs = [system_cost(s[0], int(s[1][s[0]]) if s[0] else 0) for s in systems]
    idx = partition_systems(costs, world)[rank]
    return idx, [systems[q] for q in idx]
