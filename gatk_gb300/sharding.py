"""Sharding of active regions across GPUs: regions are independent, so ranks split them with no
collective on the data path; only timings are reduced (max over ranks) for reporting."""
from __future__ import annotations

import heapq

import numpy as np


def partition_by_cells(cells_per_region, world: int) -> list[np.ndarray]:
    """Greedy longest-first assignment of regions to `world` ranks by cell count (strong scaling).
    Returns, per rank, the sorted region indices it owns; every region appears exactly once."""
    cells = np.asarray(cells_per_region, dtype=np.int64)
    order = np.argsort(-cells, kind="stable")
    heap = [(0, r) for r in range(world)]
    owned = [[] for _ in range(world)]
    for g in order:
        load, r = heapq.heappop(heap)
        owned[r].append(int(g))
        heapq.heappush(heap, (load + int(cells[g]), r))
    return [np.array(sorted(o), dtype=np.int64) for o in owned]


def block_range(n_regions_per_rank: int, rank: int) -> tuple[int, int]:
    """Weak scaling: rank r owns regions [r*n, (r+1)*n) of the generator's region sequence."""
    return rank * n_regions_per_rank, (rank + 1) * n_regions_per_rank


def reduce_max(value: float, device=None) -> float:
    """Max of a host float over all ranks of the default process group (identity without one)."""
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def reduce_sum(value: float, device=None) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()):
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())
