"""Multi-GPU layout of the path: replicas and sharded batches.

A single RBF system is solved on one GPU (the headline runs one replica per
GPU).  A batch of independent systems shards across ranks with no data-path
collective: each rank factors and solves its own systems, and only the
results are gathered.  Systems are assigned by their Cholesky / LU cost,
proportional to N^3, with the longest-processing-time-first rule, so the
ranks finish close together.  Works with any torch.distributed backend
(NCCL on GPUs, gloo for the CPU tests).
"""
from __future__ import annotations

import heapq


def shard_systems(sizes, world: int):
    """Partition system indices over `world` ranks by N^3 cost (LPT).

    Returns a list of `world` lists of indices; every index appears exactly
    once, and each list is in ascending index order.
    """
    if world < 1:
        raise ValueError("world must be >= 1")
    order = sorted(range(len(sizes)), key=lambda i: (-int(sizes[i]) ** 3, i))
    heap = [(0, r) for r in range(world)]
    heapq.heapify(heap)
    parts = [[] for _ in range(world)]
    for i in order:
        load, r = heapq.heappop(heap)
        parts[r].append(i)
        heapq.heappush(heap, (load + int(sizes[i]) ** 3, r))
    return [sorted(p) for p in parts]


def shard_imbalance(sizes, parts) -> float:
    """max rank cost / mean rank cost (1.0 = perfect balance)."""
    costs = [sum(int(sizes[i]) ** 3 for i in p) for p in parts]
    mean = sum(costs) / max(1, len(costs))
    return max(costs) / mean if mean > 0 else 1.0


def max_over_ranks(value: float, device=None) -> float:
    """Maximum of a per-rank float over the process group (itself without one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def gather_results(local: dict):
    """Gather {system index: result} dicts from every rank into one dict."""
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return dict(local)
    out = [None] * dist.get_world_size()
    dist.all_gather_object(out, local)
    merged = {}
    for part in out:
        merged.update(part)
    return merged
