"""Sharding independent sector solves over ranks (one GPU per rank).

Sectors, flux twists and served requests share nothing, so N GPUs take
disjoint shards and no collective runs on the data path; results are gathered
on the host afterwards.  ``shard`` balances estimated cost deterministically
(longest-processing-time first), so every rank computes the same assignment
without communication.
"""
from __future__ import annotations

from typing import Callable, List, Sequence, TypeVar

T = TypeVar("T")


def shard_indices(costs: Sequence[float], world: int) -> List[List[int]]:
    """Indices per rank: items sorted by decreasing cost, each given to the
    least-loaded rank (ties to the lower rank); within a rank, original order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    out: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += float(costs[i])
    return [sorted(ix) for ix in out]


def shard(items: Sequence[T], rank: int, world: int, cost: Callable[[T], float] = lambda _: 1.0) -> List[T]:
    """This rank's share of ``items``."""
    idx = shard_indices([cost(x) for x in items], world)[rank]
    return [items[i] for i in idx]
