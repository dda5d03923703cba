"""Scene sharding for replicas on several GPUs (host logic only).

Scenes of a batch are independent (no exchange step), so N processes, one
per GPU, can each build and trace a disjoint subset with no collective on the
data path.  ``partition_scenes`` splits scenes into contiguous ranges of
roughly equal work (triangles x rays)."""
from __future__ import annotations

from typing import List, Sequence, Tuple


def partition_scenes(work: Sequence[int], world: int) -> List[Tuple[int, int]]:
    """Contiguous ranges [a, b) of scene indices, one per rank, balancing the
    summed work greedily; every scene belongs to exactly one range."""
    if world < 1:
        raise ValueError("world must be >= 1")
    n = len(work)
    total = float(sum(work))
    ranges, a, acc = [], 0, 0.0
    for r in range(world):
        if r == world - 1:
            ranges.append((a, n))
            break
        target = total * (r + 1) / world
        b = a
        while b < n and (acc + work[b] <= target or b == a) and n - b > world - 1 - r:
            acc += work[b]
            b += 1
        # one more scene if that lands closer to the cumulative target
        if b < n and n - b > world - 1 - r and abs(acc + work[b] - target) < abs(acc - target):
            acc += work[b]
            b += 1
        ranges.append((a, b))
        a = b
    return ranges
