"""Instance sharding of the batched workload across ranks, one GPU per rank.

The batched configuration solves many independent SDPs (control/LMI instances with
m ~ U[20, 350] and two blocks of sizes ~ U[15, 90]).  The instances are the units of
work: they are partitioned over the ranks by estimated cost, every rank solves its own
share on its own GPU with no exchange during the solves, and the per-instance results
are gathered on rank 0 in the original order.  There is no collective on the data path;
the only cross-rank traffic is the final gather of a few numbers per instance.

Cost model: one interior-point iteration is dominated by the dense products and
factorisations of the blocks (about n_b^3 multiply-adds each) and by the Cholesky of the
m x m Schur matrix (m^3 / 3), and the iteration counts of these instances are similar,
so an instance costs about sum_b n_b^3 + m^3.
"""
from __future__ import annotations

import heapq
from typing import Callable, Sequence


def instance_cost(m: int, blocks: Sequence[int]) -> int:
    """Estimated work of one instance: sum over blocks of n_b^3, plus m^3."""
    return sum(int(n) ** 3 for n in blocks) + int(m) ** 3


def partition(costs: Sequence[int], world: int) -> list[list[int]]:
    """Split instance indices over `world` ranks, largest first onto the least loaded rank
    (ties go to the lowest rank).  Deterministic: every rank computes the same split.
    Each rank's list is returned in increasing index order."""
    if world < 1:
        raise ValueError("world must be positive")
    heap = [(0, r) for r in range(world)]
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + int(costs[i]), r))
    return [sorted(p) for p in parts]


def loads(costs: Sequence[int], parts: Sequence[Sequence[int]]) -> list[int]:
    """Summed estimated cost of each rank's instances."""
    return [sum(int(costs[i]) for i in p) for p in parts]


def solve_sharded(instances: Sequence, costs: Sequence[int], solve: Callable[[list], list], rank: int, world: int,
                  dist=None) -> list | None:
    """Solve this rank's share with `solve` (a list of instances -> a list of results, one
    each) and gather every rank's results on rank 0, returned there in the instances'
    order (None on the other ranks).  `dist` is torch.distributed (any backend with
    gather_object, e.g. gloo) or None for a single rank."""
    parts = partition(costs, world)
    mine = parts[rank]
    results = solve([instances[i] for i in mine])
    if len(results) != len(mine):
        raise RuntimeError("solve returned a different number of results than instances")
    local = list(zip(mine, results))
    if dist is None or world == 1:
        gathered = [local]
    else:
        gathered = [None] * world if rank == 0 else None
        dist.gather_object(local, gathered, dst=0)
    if rank != 0:
        return None
    out: list = [None] * len(instances)
    seen = 0
    for part in gathered:
        for i, r in part:
            out[i] = r
            seen += 1
    if seen != len(instances):
        raise RuntimeError("the gather lost instances")
    return out
