"""Scene sharding of the batched form over ranks (one GPU per rank).

The scenes of a batch are independent, so N ranks each shoot their own share
with no exchange of data: the only collectives are the bench's barrier and
max-over-ranks of the timings.  Shares are balanced by triangle count, which
is what a scene's step costs (one walk per receiver corner).
"""
from __future__ import annotations

import heapq
from typing import List, Sequence


def partition_scenes(weights: Sequence[int], world: int) -> List[List[int]]:
    """Deterministic greedy (longest first) split of scene indices over
    `world` ranks: each scene, heaviest first (ties: lower index first), goes
    to the rank with the least weight so far (ties: lower rank).  Every index
    lands in exactly one share; each share is returned in ascending order."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(weights)), key=lambda i: (-int(weights[i]), i))
    heap = [(0, r) for r in range(world)]
    shares: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + int(weights[i]), r))
    return [sorted(s) for s in shares]
