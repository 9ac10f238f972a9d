"""Autotuner front end: pick the FP32 launch shape for a workload, with an on-disk cache.

The search itself is native (``ghmm_autotune`` in libghmm.so: every candidate tuning is marshalled and timed
on the GPU with CUDA events, the fastest is set on the context).  This module chooses the sample, keys the
result by device and workload shape, and keeps it in a JSON cache so that a later process on the same kind
of GPU with the same kind of workload sets the tuning without searching again.

Cache file: ``$GHMM_TUNING_CACHE``, else ``$XDG_CACHE_HOME/gatk_gb300/tuning.json`` (``~/.cache`` when
XDG_CACHE_HOME is unset).
"""
from __future__ import annotations

import ctypes
import hashlib
import json
import os
import time

import numpy as np

from . import native
from .workload import Workload

# Cells of the autotuning sample: about 60 ms per forward on one GB300.  The sample has to carry the
# workload's load balance as well as its shapes: on workload 1 a 4e10-cell sample preferred 4,096-column
# tasks (a small batch is dominated by its last tasks), while the whole workload runs fastest with 16,384
# (271 vs 276 ms for the FP32 launch set).
SAMPLE_CELLS = 2e11
# Default candidates (rows per lane single-strip, multi-strip, haplotype columns per task): the shapes that
# won or came close on workloads 1, 2 and 4.  ghmm_autotune's built-in 18-shape grid is used when the caller
# passes candidates=[] explicitly.
DEFAULT_CANDIDATES = [(8, 8, 16384), (8, 8, 8192), (8, 8, 4096), (8, 6, 16384), (8, 4, 16384), (6, 8, 16384)]


def cache_path() -> str:
    p = os.environ.get("GHMM_TUNING_CACHE")
    if p:
        return p
    base = os.environ.get("XDG_CACHE_HOME") or os.path.join(os.path.expanduser("~"), ".cache")
    return os.path.join(base, "gatk_gb300", "tuning.json")


def _library_id() -> str:
    st = os.stat(native.lib_path())
    return f"{st.st_size}-{int(st.st_mtime)}"


def _device_id(device: int) -> str:
    try:
        import torch

        p = torch.cuda.get_device_properties(device)
        return f"{p.name}|sm{p.major}{p.minor}|{p.multi_processor_count}"
    except Exception:  # torch without CUDA: key on the ordinal only
        return f"device{device}"


def workload_signature(wl: Workload) -> str:
    """Shape of a workload as the launch shape sees it: the cell-weighted distribution of rows per lane
    (ceil(read length / 32), capped at 64) and of haplotype columns per region, in coarse bins."""
    rl = wl.read_lengths()
    hl = wl.hap_lengths()
    reg_cols = np.add.reduceat(hl, wl.region_hap_off[:-1]) if len(hl) else np.zeros(0, np.int64)
    reg_cols = np.where(np.diff(wl.region_hap_off) > 0, reg_cols, 0)
    read_region = np.repeat(np.arange(wl.n_regions), np.diff(wl.region_read_off))
    w = rl * reg_cols[read_region] if len(rl) else np.zeros(0)
    k = np.minimum((rl + 31) // 32, 64)
    hk = np.bincount(k, weights=w, minlength=65)
    hk = np.round(hk / max(hk.sum(), 1) * 20).astype(int)  # 5% bins
    cols_bin = np.minimum(np.log2(np.maximum(reg_cols, 1)).astype(int), 20)
    rc = np.bincount(cols_bin, weights=np.diff(wl.out_off), minlength=21)
    rc = np.round(rc / max(rc.sum(), 1) * 20).astype(int)
    return hashlib.sha1((",".join(map(str, hk)) + "|" + ",".join(map(str, rc))).encode()).hexdigest()[:16]


def sample(wl: Workload, cells: float = SAMPLE_CELLS) -> Workload:
    """Regions spread evenly over the workload until the sample holds about `cells` cells."""
    cpr = wl.cells_per_region()
    total = int(cpr.sum())
    if total <= cells:
        return wl
    step = max(1, int(total / cells))
    idx = np.arange(0, wl.n_regions, step)
    parts = [wl.subset(int(g), int(g) + 1) for g in idx]
    return concat(parts)


def concat(parts: list[Workload]) -> Workload:
    def offs(key):
        arrs, base = [], 0
        for i, p in enumerate(parts):
            a = getattr(p, key)
            arrs.append((a if i == 0 else a[1:]) + base)
            base += int(a[-1])
        return np.concatenate(arrs)

    cat = lambda key: np.concatenate([getattr(p, key) for p in parts])
    return Workload(region_read_off=offs("region_read_off"), region_hap_off=offs("region_hap_off"),
                    read_off=offs("read_off"), bases=cat("bases"), quals=cat("quals"), ins=cat("ins"),
                    dels=cat("dels"), gcp=cat("gcp"), hap_off=offs("hap_off"), hap_bases=cat("hap_bases"),
                    out_off=offs("out_off"))


def _load(path: str) -> dict:
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(path: str, data: dict) -> None:
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = f"{path}.{os.getpid()}.tmp"
    with open(tmp, "w") as f:
        json.dump(data, f, indent=1, sort_keys=True)
    os.replace(tmp, path)


def autotune(engine, wl: Workload, device: int = 0, use_cache: bool = True, candidates=None, reps: int = 3,
             path: str | None = None, sample_cells: float = SAMPLE_CELLS) -> dict:
    """Set the fastest tuning for workloads shaped like `wl` on `engine` and return it.

    Returns {"max_rows_per_lane", "max_rows_per_lane_multi", "chunk_cols", "cached", "key", "ms"
    (candidate -> median ms, when searched), "search_s"}.
    """
    path = path or cache_path()
    key = f"{_device_id(device)}|{_library_id()}|{workload_signature(wl)}|fp{64 if engine.double_precision else 32}"
    cache = _load(path) if use_cache else {}
    if key in cache:
        t = cache[key]
        engine.set_tuning(t["max_rows_per_lane"], t["max_rows_per_lane_multi"], t["chunk_cols"])
        return dict(t, cached=True, key=key)
    smp = sample(wl, sample_cells)
    flat = smp.as_flat()
    if candidates is None:
        candidates = DEFAULT_CANDIDATES
    if candidates:
        n = len(candidates)
        cand = (native.Tuning * n)(*[native.Tuning(*c, 0) for c in candidates])
    else:
        n = 18
        cand = None
    ms = np.zeros(n, dtype=np.float64)
    best = native.Tuning()
    t0 = time.perf_counter()
    rc = engine.L.ghmm_autotune(engine.handle, ctypes.byref(flat), cand, len(candidates) if candidates else 0,
                                reps, ctypes.byref(best), ms.ctypes.data_as(native._f64p))
    native.check(rc, engine.handle)
    search_s = time.perf_counter() - t0
    grid = candidates or [(a, b, c) for a in (8, 6, 4) for b in (8, 6, 4) for c in (16384, 4096)]
    t = {"max_rows_per_lane": best.max_rows_per_lane, "max_rows_per_lane_multi": best.max_rows_per_lane_multi,
         "chunk_cols": best.chunk_cols,
         "ms": {f"{a},{b},{c}": float(m) for (a, b, c), m in zip(grid, ms)},
         "sample_cells": int(smp.cells_per_region().sum()), "search_s": search_s}
    if use_cache:
        cache = _load(path)
        cache[key] = t
        _store(path, cache)
    return dict(t, cached=False, key=key)
