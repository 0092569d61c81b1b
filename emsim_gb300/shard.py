"""Image-parallel sharding across GPUs (one process per GPU).

Images are independent, so a batch is split across ranks with no collective on the
data path: every rank images its share and only the finished images are gathered (to
rank 0, on the host) at the end.  Shares are balanced by an estimated cost per image
(slices x pixels x log2(pixels), the FFT work of the multislice loop) with the
longest-processing-time rule, which is deterministic so every rank computes the same
partition without communicating.
"""
from __future__ import annotations

import math
from typing import Dict, List, Sequence


def image_cost(n_slices: int, n1: int, n2: int) -> float:
    px = n1 * n2
    return float(n_slices) * px * math.log2(max(px, 2))


def partition(costs: Sequence[float], world: int) -> List[List[int]]:
    """Greedy LPT: items in decreasing cost (ties by index) go to the least-loaded rank
    (ties by rank).  Each share is returned in increasing item order."""
    if world < 1:
        raise ValueError("world size must be >= 1")
    load = [0.0] * world
    shares: List[List[int]] = [[] for _ in range(world)]
    for i in sorted(range(len(costs)), key=lambda k: (-costs[k], k)):
        r = min(range(world), key=lambda q: (load[q], q))
        shares[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shares]


def my_share(costs: Sequence[float], rank: int, world: int) -> List[int]:
    return partition(costs, world)[rank]


def gather_to_root(local: Dict[int, object], n_items: int, rank: int, world: int, group=None):
    """Collect {item index: result} from every rank on rank 0 (host objects through
    torch.distributed.gather_object).  Rank 0 gets the results in item order; other
    ranks get None."""
    import torch.distributed as dist
    if world == 1:
        return [local[i] for i in range(n_items)]
    parts = [None] * world if rank == 0 else None
    dist.gather_object(local, parts, dst=0, group=group)
    if rank != 0:
        return None
    merged: Dict[int, object] = {}
    for p in parts:
        merged.update(p)
    missing = [i for i in range(n_items) if i not in merged]
    if missing:
        raise RuntimeError(f"images missing after gather: {missing[:10]}")
    return [merged[i] for i in range(n_items)]
