"""Instance sharding of an ensemble across ranks (one process per GPU).

Independent Schroedinger instances need no exchange while they are advanced,
so the multi-GPU form of an ensemble is a partition of the instances: every
rank builds a ``Batch`` of its own share, runs it, and the per-instance
results (convergence flag, steps taken, inner iterations, final M-norm) are
gathered to rank 0 at the end.  The only collectives are that gather and the
timing barrier; nothing crosses ranks on the data path.

The partition is deterministic (the same on every rank, computed from the
instances alone): longest-processing-time order by cost (element-local nodes
times an iteration weight), each instance to the rank with the least load so
far, ties to the lower rank.  For 1,024 instances of 16..1,024 elements it
balances the load within a few percent.
"""
from __future__ import annotations

from typing import Callable, Sequence


def instance_cost(n_elements: int, p: int) -> float:
    """relative cost of one instance-step: element-local nodes times the
    iteration growth with the degree (the element preconditioner keeps the
    count nearly mesh independent, so only the node count and a mild degree
    factor remain)"""
    N = p + 1
    return float(n_elements * N * N) * (1.0 + 0.05 * p)


def shard(costs: Sequence[float], world: int) -> list[list[int]]:
    """indices of the instances of every rank (each list ascending)"""
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    load = [0.0] * world
    parts: list[list[int]] = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        parts[r].append(i)
        load[r] += float(costs[i])
    return [sorted(p) for p in parts]


def imbalance(costs: Sequence[float], parts: list[list[int]]) -> float:
    """max rank load / mean rank load (1.0 is perfect balance)"""
    loads = [sum(float(costs[i]) for i in p) for p in parts]
    mean = sum(loads) / len(loads) if loads else 0.0
    return max(loads) / mean if mean > 0 else 1.0


def gather_results(local: dict, n_total: int, rank: int, world: int, dist=None):
    """collect {instance index: result} of every rank on rank 0, ordered by
    instance index; other ranks get None.  With world == 1 (or no
    process group) the local results are returned."""
    if world == 1 or dist is None:
        return [local[i] for i in range(n_total)]
    obj = [None] * world if rank == 0 else None
    dist.gather_object(local, obj, dst=0)
    if rank != 0:
        return None
    merged: dict = {}
    for part in obj:
        dup = set(merged) & set(part)
        if dup:
            raise RuntimeError(f"instances reported by two ranks: {sorted(dup)[:5]}")
        merged.update(part)
    missing = [i for i in range(n_total) if i not in merged]
    if missing:
        raise RuntimeError(f"instances missing from the gather: {missing[:5]}")
    return [merged[i] for i in range(n_total)]


def run_sharded(costs: Sequence[float], rank: int, world: int, run_share: Callable[[list[int]], dict], dist=None):
    """run this rank's share (run_share(indices) -> {index: result}) and
    gather every rank's results on rank 0"""
    mine = shard(costs, world)[rank]
    local = run_share(mine) if mine else {}
    if set(local) != set(mine):
        raise RuntimeError("run_share must return one result per instance of the share")
    return gather_results(local, len(costs), rank, world, dist)
