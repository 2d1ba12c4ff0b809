"""Instance sharding across ranks (one process per GPU).

Magnus instances are independent, so a batch shards by instance with no
collective during the computation: each rank runs its share through the
engine and one gather at the end returns every instance's result in the
caller's order.  Shares balance the cost model of the chunk kernels,
(n - 1) * S * d^3 flops plus the prefix passes' S * n * d^2 per instance
(largest-first greedy assignment).  Every run here has one GPU, so the
engine's benchmarks run replicas; this module is the host side of a
multi-GPU batch and is tested with gloo ranks on the CPU.
"""
from __future__ import annotations

import heapq
from typing import Callable, Dict, List, Sequence


def instance_cost(d: int, samples: int, n: int) -> float:
    """Work model of one instance: chunk-kernel products and prefix passes."""
    return float(max(n - 1, 0)) * samples * d ** 3 + float(samples) * n * d * d


def partition(costs: Sequence[float], world: int) -> List[List[int]]:
    """Indices per rank (each list ascending), balancing the summed cost by
    largest-first greedy assignment to the least-loaded rank."""
    if world < 1:
        raise ValueError("world must be at least 1")
    heap = [(0.0, r) for r in range(world)]
    shares: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        load, r = heapq.heappop(heap)
        shares[r].append(i)
        heapq.heappush(heap, (load + float(costs[i]), r))
    return [sorted(s) for s in shares]


def gather(local: Dict[int, object], group=None) -> Dict[int, object]:
    """Merge every rank's {index: result} (torch.distributed all_gather_object;
    the only exchange of a sharded batch)."""
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized():
        return dict(local)
    parts: List[Dict[int, object]] = [None] * dist.get_world_size(group)  # type: ignore[list-item]
    dist.all_gather_object(parts, local, group=group)
    merged: Dict[int, object] = {}
    for p in parts:
        merged.update(p)
    return merged


def sharded_map(fn: Callable[[List[int]], Dict[int, object]], costs: Sequence[float], rank: int, world: int,
                group=None) -> List[object]:
    """Run fn on this rank's share (fn maps a list of instance indices to
    {index: result}, e.g. one batched engine call), gather, and return all
    results in instance order."""
    share = partition(costs, world)[rank]
    local = fn(share) if share else {}
    merged = gather(local, group) if world > 1 else dict(local)
    return [merged[i] for i in range(len(costs))]
