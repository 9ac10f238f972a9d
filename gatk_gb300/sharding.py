"""Sharding of active regions across GPUs: pairs are independent, so ranks split them with no
collective on the data path; only timings are reduced (max over ranks) for reporting.

Strong scaling uses the library's own split (ghmm_multi_plan, the split ghmm_multi_compute_regions applies
within one process): reads numbered in region order are cut into one contiguous range per device of about
equal cells, and each range owns a contiguous slice of the read-major output."""
from __future__ import annotations

import ctypes

import numpy as np

from . import native


def read_slices(wl, world: int) -> list[dict]:
    """Per rank: {read_begin, read_end, out_begin, out_end, cells} of the workload's strong-scaling split."""
    regs = wl.as_regions()
    sl = (native.MultiSlice * world)()
    native.check(native.lib().ghmm_multi_plan(ctypes.cast(regs, ctypes.c_void_p), wl.n_regions, world, sl))
    return [{k: int(getattr(s, k)) for k, _ in native.MultiSlice._fields_} for s in sl]


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
