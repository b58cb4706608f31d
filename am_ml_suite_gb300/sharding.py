"""Partition of independent problems over ranks (one process per GPU).

Batched workloads shard by problem with no exchange step: each rank runs its
share as one batch.  Problems are assigned longest-processing-time first: in
decreasing cost order, each goes to the rank with the least cost so far (ties to
the lower rank), so every rank computes the same partition without
communicating."""
from __future__ import annotations

from typing import List, Sequence


def problem_cost(shape: Sequence[int]) -> float:
    """Relative cost of one SIMP iteration of an nx*ny*nz problem: elements times
    the growth of Jacobi-PCG iterations with the grid's longest edge."""
    nx, ny, nz = (int(v) for v in shape)
    return float(nx * ny * nz) * float(max(nx, ny, nz))


def partition(costs: Sequence[float], world: int) -> List[List[int]]:
    """Indices of the problems of each rank (each list ascending)."""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]
