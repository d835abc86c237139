"""Instance sharding across ranks (one process per GPU).

Triples of a ragged batch are independent, so N ranks split the instances with no
data-path collective: a greedy longest-processing-time split of the per-instance cost
(amplitudes x (D + 1) recurrence terms).  Each rank plans and runs its own share
(weak scaling); results stay on the rank that computed them.
"""

from __future__ import annotations

import heapq

import numpy as np


def instance_costs(shapes) -> np.ndarray:
    return np.array([int(np.prod(s)) * (len(s) + 1) for s in shapes], np.int64)


def shard_instances(costs, world_size: int) -> list[list[int]]:
    """Split instance indices over `world_size` ranks, largest cost first to the least-loaded rank."""
    costs = np.asarray(costs)
    if world_size <= 1:
        return [list(range(len(costs)))]
    order = np.argsort(-costs, kind="stable")
    heap = [(0, r) for r in range(world_size)]
    parts: list[list[int]] = [[] for _ in range(world_size)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(int(i))
        heapq.heappush(heap, (load + int(costs[i]), r))
    return [sorted(p) for p in parts]


def local_instances(costs, rank: int, world_size: int) -> list[int]:
    return shard_instances(costs, world_size)[rank]
