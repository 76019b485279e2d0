"""Work placement across GPUs for the many-scene workloads: one process per GPU, every scene
whole on one GPU, no data exchanged between them.

The reference runs one world per process and has no placement of its own; this module decides
which GPU takes which scene of a batch or which job of a stream, by the work a scene costs:
spheres x steps.

* `pack_scenes` — a fixed batch (every scene known up front): longest processing time first,
  each scene to the GPU with the least work so far.
* `dispatch_stream` — jobs in arrival order, each to the GPU with the least work handed out so
  far (what a front end that sees one job at a time can do).

Both are deterministic: ties go to the lower scene index and the lower rank, so every process
computes the same placement from the same list without communicating.
"""
from __future__ import annotations

import heapq
from typing import List, Sequence


def _check(weights: Sequence[float], ranks: int) -> None:
    if ranks < 1:
        raise ValueError("ranks must be at least 1")
    for w in weights:
        if not (w >= 0.0):
            raise ValueError(f"scene weight {w!r} is not a non-negative number")


def pack_scenes(weights: Sequence[float], ranks: int) -> List[List[int]]:
    """Scene indices per rank (each list ascending): scenes in decreasing weight go one by one
    to the rank with the least total weight so far.  The heaviest rank carries at most the
    average plus the heaviest scene (and at most 4/3 of the best possible largest load)."""
    _check(weights, ranks)
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    heap = [(0.0, r) for r in range(ranks)]
    out: List[List[int]] = [[] for _ in range(ranks)]
    for i in order:
        load, r = heapq.heappop(heap)
        out[r].append(i)
        heapq.heappush(heap, (load + float(weights[i]), r))
    for lst in out:
        lst.sort()
    return out


def dispatch_stream(weights: Sequence[float], ranks: int) -> List[int]:
    """The rank of each job of a stream, in arrival order: each job goes to the rank with the
    least total weight handed out before it."""
    _check(weights, ranks)
    heap = [(0.0, r) for r in range(ranks)]
    out: List[int] = []
    for w in weights:
        load, r = heapq.heappop(heap)
        out.append(r)
        heapq.heappush(heap, (load + float(w), r))
    return out


def loads(weights: Sequence[float], parts: List[List[int]]) -> List[float]:
    """Total weight per rank of a placement."""
    return [float(sum(weights[i] for i in p)) for p in parts]
