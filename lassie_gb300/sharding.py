"""Instance sharding across GPUs (one process per GPU).

Instances are independent, so sharding needs no data-path collective: each
rank integrates its own instances; the only exchanges are the host-side
max of the elapsed time and, optionally, the gather of trajectories.
"""
from __future__ import annotations

from typing import List, Sequence


def weak_shard(n_per_rank: int, rank: int) -> range:
    """Instance ids of `rank` when every rank owns `n_per_rank` instances."""
    return range(rank * n_per_rank, (rank + 1) * n_per_rank)


def cost_shard(sizes: Sequence[int], world: int) -> List[List[int]]:
    """Split one fixed batch over `world` ranks, balancing the dense-LU cost
    (N^3) greedily, largest first.  Returns the instance ids of each rank."""
    order = sorted(range(len(sizes)), key=lambda q: -sizes[q])
    load = [0.0] * world
    parts: List[List[int]] = [[] for _ in range(world)]
    for q in order:
        r = min(range(world), key=lambda w: (load[w], w))
        parts[r].append(q)
        load[r] += float(sizes[q]) ** 3
    return [sorted(p) for p in parts]


def max_over_ranks(value: float) -> float:
    """Max of a host scalar over the default process group (identity without
    one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    """Sum of a host scalar over the default process group (identity without
    one)."""
    import torch
    import torch.distributed as dist
    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return value
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
