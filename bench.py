#!/usr/bin/env python
"""PairHMM read-likelihood benchmark on GB300: GCUPS of the batched FP32 + FP64-rerun forward.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload 1]
    python bench.py --stream [--regions N] [--batch-cells C]     (workload 4 through the streaming queue)
    python bench.py --calib                                      (workload 3: calibration forward + backward)
    python bench.py --pd [--regions N]                           (PD-HMM, DRAGEN-GATK mode)
    python bench.py --sw [--regions N] [--workload 2]            (Smith-Waterman realignment to the best haplotype)

A step is one forward over the whole workload (default: workload 1, 10,000 synthetic active regions,
seed 1, ~1.06e12 cells): every read x haplotype pair of every region, FP32 wavefront plus the FP64 rerun
of every pair whose FP32 result underflows.  `value` is GCUPS (cells / device second) with the inputs
already resident in HBM, timed with CUDA events on the library's stream; `e2e` is the same metric
through the JNI-shaped C-ABI call (ghmm_compute_regions) from host buffers: marshalling, H2D copies,
kernels, D2H of the results and their validation are all inside its timed region.

Beside it the line reports the plain FP64 kernel (one pair per thread block, one launch per region) on a
subsample, the accuracy of the timed results against the FP64 oracle on the CPU-baseline sample, the
roofline of the dominant kernel (the FP32 bucket launches) against the FP32 FMA-pipe peak measured in the
same run, and the FP64 oracle's GCUPS on the host cores.

--impl reference times the reference's algorithm on the host CPU: the FP64 restatement of
LoglessPairHMM (oracle/, OpenMP over pairs on every host core) on a bounded sample of the same workload;
GATK's Java and GKL's AVX code cannot run on this machine (no JVM; GKL is x86-only).
Under torchrun with N > 1 each rank runs its own 10,000 regions on its own GPU (weak scaling; the regions
are independent so no collective touches the data path), or with --scaling strong its share of one workload as the
library's multi-device split (ghmm_multi_plan) cuts it; rank 0 prints.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "PairHMM GCUPS, batched FP32 vs plain FP64 on 1 GB300 at |Δlog10 L|≤1e-3"
FLOP_PER_CELL = 11  # M: add, mul, fma, mul (5); I: fma (3); D: fma (3); FMA counted as 2
CPU_SAMPLE_CELLS = 2.0e10  # cells of the oracle's timed sample (about 5-15 s on 16 cores)
PLAIN_SAMPLE_CELLS = 2.0e10  # cells of the plain-FP64-kernel comparison


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock and throttle reasons)."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.device)], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=5)
        sm, mx, pw, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
                pw.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "power_w_max": max(pw) if pw else None, "reasons": sorted(reasons), "samples": len(sm)}


def cpu_sample(wl, cells_target):
    """Leading regions of the workload whose cells reach cells_target (the deterministic CPU sample)."""
    import numpy as np

    cpr = wl.cells_per_region()
    n = int(np.searchsorted(np.cumsum(cpr), cells_target)) + 1
    n = max(1, min(n, wl.n_regions))
    return n, int(cpr[:n].sum())


def run_reference(args):
    """--impl reference: the FP64 oracle (LoglessPairHMM restated in C, OpenMP) on host cores."""
    rank, world, _ = dist_env()
    if rank != 0:
        return 0
    from gatk_gb300 import workload as W
    from oracle import oracle as O

    wl_full = W.generate(args.workload, regions=args.regions or None)
    n, cells = cpu_sample(wl_full, args.cpu_cells)
    sub = wl_full.subset(0, n)
    threads = O.num_threads()
    times = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        O.compute_workload(sub, threads=0)
        dt = time.perf_counter() - t0
        if i >= args.warmup:
            times.append(dt)
    gcups = cells / statistics.mean(times) / 1e9
    sample = (f"first {n} of {wl_full.n_regions} regions of workload {args.workload} ({cells:.3e} cells, "
              f"{sub.n_pairs} pairs) per step")
    line = {
        "impl": "reference", "metric": METRIC, "value": gcups, "unit": "GCUPS", "higher_is_better": True,
        "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": statistics.mean(times) * 1e3, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (deterministic generator, seed per workload)",
        "config": workload_config(args, wl_full),
        "cpu_baseline": {"value": gcups, "unit": "GCUPS", "cores": threads, "kind": "port", "sample": sample,
                         "host": f"{platform.machine()} x{os.cpu_count()}"},
        "e2e": {"value": gcups, "unit": "GCUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": ("FP64 C restatement of LoglessPairHMM (oracle/pairhmm_oracle.c); GATK's Java LoglessPairHMM needs "
                 "a JVM and GKL AVX_LOGLESS_CACHING_OMP is x86-only, neither runs on this host"),
    }
    print(json.dumps(line), flush=True)
    return 0


def workload_config(args, wl):
    names = {0: "workload 0: 1 region, 8 haps x 64 reads, seed 0",
             1: "workload 1: 10,000 active regions, seed 1 (haps U[2,32] of U[200,600] bp, "
                "reads lognormal(4,1) of U[100,250] bp)",
             2: "workload 2: 2,000 long-pair regions, seed 2", 4: "workload 4 body: workload 1 distributions, seed 4"}
    return {"workload": names.get(args.workload, f"workload {args.workload}"), "regions": wl.n_regions,
            "pairs": wl.n_pairs, "cells": int(wl.cells_per_region().sum()),
            "l2": f"inputs larger than L2 ({(wl.bases.nbytes * 5 + wl.hap_bases.nbytes) / 1e6:.0f} MB of read and "
                  f"haplotype bytes vs 129 MB L2)"}


def run_ours(args):
    import numpy as np
    import torch

    from gatk_gb300 import native, workload as W
    from gatk_gb300.pairhmm import Engine

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    torch.cuda.set_device(local)
    device = local

    def barrier():
        if dist is not None:
            dist.barrier()

    from gatk_gb300 import sharding

    def max_over_ranks(x: float) -> float:
        return sharding.reduce_max(x, device=f"cuda:{device}")

    def sum_over_ranks(x: float) -> float:
        return sharding.reduce_sum(x, device=f"cuda:{device}")

    eng = Engine(device=device)
    peaks = eng.measure_peaks()
    n_regions = args.regions or int(native.synth_lib().ghmm_synth_default_regions(args.workload))
    if args.scaling == "strong":
        # strong scaling: one workload, cut by the library's split (ghmm_multi_plan) into one read range per rank
        wl_all = W.generate(args.workload, regions=n_regions)
        mine = sharding.read_slices(wl_all, world)[rank]
        wl = wl_all.read_slice(mine["read_begin"], mine["read_end"])
        del wl_all
    else:
        # weak scaling: every rank owns its own block of regions of the same distribution
        g0, g1 = sharding.block_range(n_regions, rank)
        wl = W.generate(args.workload, regions=g1 - g0, region_begin=g0)
    cells = int(wl.cells_per_region().sum())
    tuning = apply_tuning(args, eng, wl)

    # ---- device-resident forward (value) ----
    batch = eng.batch(wl)
    for _ in range(args.warmup):
        batch.forward(native.MODE_FP32_RERUN)
    stream = torch.cuda.ExternalStream(eng.stream_handle(), device=f"cuda:{device}")
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    clocks = ClockSampler(device)
    clocks.start()
    barrier()
    torch.cuda.synchronize(device)
    ev0.record(stream)
    st_steps = []
    for _ in range(args.steps):
        batch.forward(native.MODE_FP32_RERUN)
        st_steps.append(batch.stats())
    ev1.record(stream)
    torch.cuda.synchronize(device)
    barrier()
    clk = clocks.stop()
    ms_step_local = ev0.elapsed_time(ev1) / args.steps
    ms_step = max_over_ranks(ms_step_local)
    total_cells = sum_over_ranks(float(cells))
    value = total_cells / (ms_step * 1e-3) / 1e9
    launches = sum(s["n_launches"] for s in st_steps)
    st = st_steps[-1]
    ms_fp32 = statistics.mean(s["ms_fp32"] for s in st_steps)
    ms_fp64 = statistics.mean(s["ms_fp64"] for s in st_steps)
    results = batch.results()
    io = batch.stats()  # byte counts of upload + forward + results (what one e2e call moves)
    rerun_frac = st["n_rerun"] / max(1, st["n_pairs"])

    # ---- e2e through the JNI-shaped C-ABI from host buffers ----
    e2e = None
    if not args.no_e2e:
        regs = wl.as_regions()
        out = np.empty(wl.n_pairs, dtype=np.float64)
        L = eng.L
        for _ in range(max(1, min(args.warmup, 2))):
            native.check(L.ghmm_compute_regions(eng.handle, regs, wl.n_regions, out.ctypes.data_as(native._f64p)),
                         eng.handle)
        barrier()
        torch.cuda.synchronize(device)
        t0 = time.perf_counter()
        e2e_steps = args.steps  # as many calls as the device-resident value times
        for _ in range(e2e_steps):
            native.check(L.ghmm_compute_regions(eng.handle, regs, wl.n_regions, out.ctypes.data_as(native._f64p)),
                         eng.handle)
        torch.cuda.synchronize(device)
        dt = (time.perf_counter() - t0) / e2e_steps
        barrier()
        dt = max_over_ranks(dt)
        same = bool(np.array_equal(out, results))
        e2e = {"value": total_cells / dt / 1e9, "unit": "GCUPS", "ms_per_step": dt * 1e3, "steps": e2e_steps,
               "h2d_bytes_per_step": int(io["h2d_bytes"]), "d2h_bytes_per_step": int(io["d2h_bytes"]),
               "api": "ghmm_compute_regions (per-read pointer arrays, as the JNI binding passes them)",
               "matches_device_resident_results": same}

    # ---- the whole workload against the GPU's FP64 mode (every pair in FP64, pinned to the oracle at 1e-9) ----
    full_fp64 = None
    if not args.no_full_check:
        batch.forward(native.MODE_FP64)
        st64 = batch.stats()
        res64 = batch.results()
        dd = absdiff(results, res64)
        full_fp64 = {"pairs": int(len(dd)), "max_abs_dlog10": float(dd.max()), "median_abs_dlog10": float(np.median(dd)),
                     "pairs_above_1e-3": int((dd > 1e-3).sum()), "pairs_above_1e-5": int((dd > 1e-5).sum()),
                     "fp64_mode_ms": st64["ms_total"], "fp64_mode_gcups": cells / (st64["ms_total"] * 1e-3) / 1e9,
                     "budget": 1e-3,
                     "what": "every FP32 + FP64-rerun result of the timed forward against the same batch in "
                             "GHMM_MODE_FP64 (all pairs in the FP64 kernel)"}

    if rank != 0:
        batch.close()
        eng.close()
        if dist is not None:
            dist.destroy_process_group()
        return 0

    # ---- accuracy and CPU baseline on the deterministic sample ----
    from oracle import oracle as O

    # the sample: leading and trailing regions of the timed workload, half the CPU cells each
    head_n, head_cells = cpu_sample(wl, args.cpu_cells / 2)
    cpr = wl.cells_per_region()
    tail_n = int(np.searchsorted(np.cumsum(cpr[::-1]), args.cpu_cells / 2)) + 1
    tail_n = max(0, min(tail_n, wl.n_regions - head_n))
    spans = [(0, head_n)] + ([(wl.n_regions - tail_n, wl.n_regions)] if tail_n else [])
    # plus the regions holding the lowest results of the timed forward: the exact FP64 tier's pairs (log10 L < -560,
    # and -Infinity where the reference's 2^1020 scale underflows too), when the workload has any
    region_of_out = np.repeat(np.arange(wl.n_regions), np.diff(wl.out_off))
    extra = []
    for mask in (np.isneginf(results), results < native.FP64_RESCALED_FLOOR):
        idx = np.nonzero(mask)[0]
        if len(idx):
            g = int(region_of_out[idx[np.argmin(results[idx]) if not np.isneginf(results[idx]).all() else 0]])
            if not any(a <= g < b for a, b in spans) and g not in extra:
                extra.append(g)
    spans += [(g, g + 1) for g in extra]
    refs, gots, cpu_dt, cpu_cells, sample_pairs = [], [], 0.0, 0, 0
    for g0, g1 in spans:
        sub = wl.subset(g0, g1)
        t0 = time.perf_counter()
        refs.append(O.compute_workload(sub, threads=0))
        cpu_dt += time.perf_counter() - t0
        gots.append(results[int(wl.out_off[g0]):int(wl.out_off[g1])])
        cpu_cells += int(cpr[g0:g1].sum())
        sample_pairs += sub.n_pairs
    ref, got = np.concatenate(refs), np.concatenate(gots)
    d = absdiff(got, ref)
    under = ref < -64.2
    accuracy = {"sample_pairs": int(sample_pairs), "max_abs_dlog10": float(d.max()),
                "median_abs_dlog10": float(np.median(d)),
                "regions": f"{head_n} leading and {tail_n} trailing regions of {wl.n_regions}"
                           + (f", and regions {extra} (the timed forward's lowest results)" if extra else ""),
                "fp64_rerun_pairs_in_sample": int(under.sum()),
                "max_abs_dlog10_fp64_reruns": float(d[under].max()) if under.any() else None,
                "exact_tier_pairs_in_sample": int((ref < native.FP64_RESCALED_FLOOR).sum()),
                "max_abs_dlog10_exact_tier": (float(d[ref < native.FP64_RESCALED_FLOOR].max())
                                              if (ref < native.FP64_RESCALED_FLOOR).any() else None),
                "neg_inf_pairs_in_sample": int(np.isneginf(ref).sum())}
    if full_fp64 is not None:
        d64 = absdiff(np.concatenate([res64[int(wl.out_off[g0]):int(wl.out_off[g1])] for g0, g1 in spans]), ref)
        full_fp64["fp64_mode_vs_oracle_on_sample_max_abs_dlog10"] = float(d64.max())
    cpu_baseline = {"value": cpu_cells / cpu_dt / 1e9, "unit": "GCUPS", "cores": O.num_threads(), "kind": "port",
                    "sample": f"first {head_n} and last {tail_n} regions of the timed workload ({cpu_cells:.3e} cells, "
                              f"{sample_pairs} pairs)",
                    "host": f"{platform.machine()} x{os.cpu_count()}"}

    # ---- plain FP64 kernel, one pair per block, one launch per region ----
    n_pl, pl_cells = cpu_sample(wl, args.plain_cells)
    with eng.batch(wl.subset(0, n_pl)) as pb:
        pb.forward(native.MODE_PLAIN_FP64)
        pb.forward(native.MODE_PLAIN_FP64)
        pst = pb.stats()
        plain_res = pb.results()
    plain_gcups = pl_cells / (pst["ms_plain"] * 1e-3) / 1e9
    plain_vs_ours = float(absdiff(plain_res, results[:len(plain_res)]).max())

    # ---- roofline of the dominant kernel: the FP32 bucket launches of one forward ----
    direct_cells = int(st["n_cells_fp64_direct"])  # pairs routed straight to FP64 (none on workload 1)
    fp32_cells = cells - direct_cells
    achieved = FLOP_PER_CELL * fp32_cells / (ms_fp32 * 1e-3) / 1e12
    peak = max(peaks["fp32_tflops"], peaks["fp32x2_tflops"])
    # the same peak from the clock: SMs x 128 FP32 lanes x 2 FLOP per FMA x the median SM clock of the timed region
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    clock_peak = sms * 128 * 2 * clk["sm_mhz"] * 1e6 / 1e12 if clk.get("sm_mhz") else None
    traffic = read_profile_traffic()
    line = {
        "metric": METRIC, "value": value, "unit": "GCUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": args.scaling,
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (deterministic generator; seeded stand-in for HaplotypeCaller active regions)",
        "config": workload_config(args, wl),
        "roofline": {"bound": "fp32_fma_pipe", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "traffic_source": "profiles (scaled): ncu dram bytes of a 2,000-region capture of the same "
                                       "kernels, scaled by cells to the full launch set",
                     "kernel": "fp32_bucket_kernel (all rows-per-lane buckets of one forward)",
                     "flop_per_cell": FLOP_PER_CELL, "cells_per_launch_set": fp32_cells,
                     "ms_per_launch_set": ms_fp32,
                     "peak_source": ("measured in this run: FFMA and FFMA2 register loops over all SMs "
                                     f"({peaks['fp32_tflops']:.1f} / {peaks['fp32x2_tflops']:.1f} TFLOP/s); "
                                     "MEASURED_PEAKS.json carries no FP32 figure"),
                     "peak_from_clock": clock_peak,
                     "frac_vs_peak_from_clock": achieved / clock_peak if clock_peak else None,
                     "peak_from_clock_source": f"{sms} SMs x 128 FP32 lanes x 2 FLOP x median SM clock of the timed "
                                               "region"},
        "cpu_baseline": cpu_baseline,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk,
        "fp64_rerun": {"pairs": int(st["n_rerun"]), "fraction": rerun_frac, "ms": ms_fp64,
                       "direct_pairs": int(st["n_fp64_direct"]), "direct_cells": direct_cells,
                       "exact_tier_pairs": int(st["n_fp64_exact"])},
        "tuning": tuning,
        "plain_fp64": {"value": plain_gcups, "unit": "GCUPS", "regions": n_pl, "cells": pl_cells,
                       "launches": int(pst["n_launches"]), "speedup_batched_vs_plain": value / world / plain_gcups,
                       "max_abs_diff_vs_batched": plain_vs_ours},
        "accuracy_vs_fp64_oracle": accuracy,
        "accuracy_vs_gpu_fp64_full_workload": full_fp64,
        "peaks_measured": peaks,
    }
    print(json.dumps(line), flush=True)
    batch.close()
    eng.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


def run_stream(args):
    """--stream: a HaplotypeCaller-shaped stream (default workload 4: 100,000 regions of workload 1's
    distributions with a 5% tail of 2,000-read x 64-haplotype regions) pushed one region at a time through
    the queue (ghmm_queue_push), then flushed.  The timed region runs from the first push to the return of
    the flush, so host copies, marshalling, H2D, kernels, D2H and delivery into the caller's arrays are all
    inside it: `value` and `e2e` are the same wall-clock GCUPS."""
    import numpy as np

    from gatk_gb300 import native, sharding, workload as W
    from gatk_gb300.pairhmm import Engine

    rank, world, local = dist_env()
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    else:
        dist = None
    eng = Engine(device=local)
    peaks = eng.measure_peaks()
    n_regions = args.regions or int(native.synth_lib().ghmm_synth_default_regions(args.workload))
    g0, g1 = sharding.block_range(n_regions, rank)
    blocks = []  # (workload, region struct addresses, output array, output addresses, mapping qualities)
    t_gen = time.perf_counter()
    block = 5000
    for a in range(g0, g1, block):
        wl = W.generate(args.workload, regions=min(block, g1 - a), region_begin=a)
        mapq = None
        if args.raw:  # the generator's qualities and 45s as raw base qualities and BI / BD tags, seeded MAPQs
            mapq = np.random.default_rng(1000 + a).integers(20, 70, size=wl.n_reads)
            base = W.as_raw_regions(wl, mapq, True)
            regs = wl
        else:
            regs = wl.as_regions()
            base = ctypes_addr(regs)
        out = np.empty(max(wl.n_pairs, 1), dtype=np.float64)
        ra = base + np.arange(wl.n_regions, dtype=np.int64) * 32
        oa = np.where(np.diff(wl.out_off) > 0, out.ctypes.data + wl.out_off[:-1] * 8, 0)
        blocks.append((wl, regs, out, ra.tolist(), oa.tolist(), mapq))
    t_gen = time.perf_counter() - t_gen
    cells = sum(int(b[0].cells_per_region().sum()) for b in blocks)
    pairs = sum(b[0].n_pairs for b in blocks)
    L = eng.L
    raw_kw = {}
    if args.raw == "pcr":
        raw_kw = {"pcr_rate_factor": 3.0}
    elif args.raw == "dragstr":
        raw_kw = {"dragstr": _prep_tables()}
    q = eng.raw_queue(blocks[0][0], int(args.batch_cells), **raw_kw) if args.raw else eng.queue(int(args.batch_cells))
    push = L.ghmm_queue_push_raw if args.raw else L.ghmm_queue_push

    def push_block(b, limit=None):
        ra, oa = b[3], b[4]
        n = len(ra) if limit is None else min(limit, len(ra))
        for g in range(n):
            rc = push(q.h, ra[g], 1, oa[g] or None)
            if rc:
                native.check(rc, eng.handle)

    # warm-up: the first regions of the first block, three times (kernels loaded, slot buffers grown)
    for _ in range(args.warmup):
        push_block(blocks[0], 1500)
        q.flush()
    before = q.info()
    clocks = ClockSampler(local)
    clocks.start()
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    for b in blocks:
        push_block(b)
    q.flush()
    dt = time.perf_counter() - t0
    clk = clocks.stop()
    after = q.info()
    info = {k: after[k] - before[k] for k in after}
    dt = sharding.reduce_max(dt, device=f"cuda:{local}") if dist is not None else dt
    total_cells = sharding.reduce_sum(float(cells), device=f"cuda:{local}") if dist is not None else float(cells)
    gcups = total_cells / dt / 1e9
    if rank != 0:
        q.close()
        eng.close()
        dist.destroy_process_group()
        return 0
    # accuracy + CPU baseline on the leading body regions of the first block
    from oracle import oracle as O

    wl0, _, out0 = blocks[0][0], blocks[0][1], blocks[0][2]
    n_cpu, cpu_cells = cpu_sample(wl0, args.cpu_cells / 20 if args.raw else args.cpu_cells)
    sub = wl0.subset(0, n_cpu)
    if args.raw:  # the oracle's own preparation of the raw reads (untimed), then its forward
        sub = _oracle_prepared(sub, blocks[0][5][:sub.n_reads], raw_kw)
    t1 = time.perf_counter()
    ref = O.compute_workload(sub, threads=0)
    cpu_dt = time.perf_counter() - t1
    d = absdiff(out0[:sub.n_pairs], ref)
    # the high-depth tail (2,000 reads x 64 haplotypes): the first two such regions of the stream, checked apart
    tail = None
    if args.workload == 4 and not args.raw:
        nr, nh = np.diff(wl0.region_read_off), np.diff(wl0.region_hap_off)
        tail_regions = [int(g) for g in np.nonzero((nr == 2000) & (nh == 64))[0][:2]]
        if tail_regions:
            dts = []
            for g in tail_regions:
                tsub = wl0.subset(g, g + 1)
                tref = O.compute_workload(tsub, threads=0)
                dts.append(absdiff(out0[int(wl0.out_off[g]):int(wl0.out_off[g + 1])], tref))
            dt_all = np.concatenate(dts)
            tail = {"regions": tail_regions, "pairs": int(len(dt_all)),
                    "cells": int(wl0.cells_per_region()[tail_regions].sum()),
                    "max_abs_dlog10": float(dt_all.max()), "median_abs_dlog10": float(np.median(dt_all))}
    fp32_cells = cells - info["n_cells_fp64_direct"]
    achieved = FLOP_PER_CELL * fp32_cells / dt / 1e12
    peak = max(peaks["fp32_tflops"], peaks["fp32x2_tflops"])
    line = {
        "metric": METRIC, "value": gcups, "unit": "GCUPS", "n_gpus": world, "steps": 1, "warmup": args.warmup,
        "ms_per_step": dt * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (deterministic generator; seeded stand-in for a HaplotypeCaller region stream)",
        "config": {"workload": (("workload 4: 100,000 regions of workload 1's distributions with a 5% tail of "
                                 "2,000 reads x 64 haplotypes, seed 4, streamed one region per push")
                                if args.workload == 4 else f"workload {args.workload}, streamed one region per push")
                   + (f"; raw reads prepared on the device ({args.raw} imputation, seeded MAPQ 20-69)"
                      if args.raw else ""),
                   "regions": g1 - g0, "pairs": pairs, "cells": cells, "batch_cells": int(args.batch_cells),
                   "l2": "inputs larger than L2 (streamed from host memory)"},
        "roofline": {"bound": "fp32_fma_pipe", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                     "frac": achieved / peak, "traffic": None,
                     "kernel": "whole stream: FP32 cells x 11 FLOP over wall-clock time (a lower bound for the kernels)",
                     "flop_per_cell": FLOP_PER_CELL},
        "e2e": {"value": gcups, "unit": "GCUPS", "ms_per_step": dt * 1e3, "h2d_bytes_per_step": int(info["h2d_bytes"]),
                "d2h_bytes_per_step": int(info["d2h_bytes"]),
                "api": ("ghmm_queue_push_raw" if args.raw else "ghmm_queue_push")
                + " per region + ghmm_queue_flush (host arrays in, host results out)"},
        "gpu_launches": int(info["n_launches"]),
        "clocks": clk,
        "queue": {"batches": int(info["n_batches"]), "device_ms_fp32_summed": info["ms_fp32"],
                  "device_ms_fp64_summed": info["ms_fp64"], "host_ms_marshal": info["ms_host_marshal"],
                  "host_ms_tasks": info["ms_host_tasks"], "generate_s_untimed": t_gen},
        "fp64_rerun": {"pairs": int(info["n_rerun"]), "fraction": info["n_rerun"] / max(1, info["n_pairs"]),
                       "direct_pairs": int(info["n_fp64_direct"])},
        "cpu_baseline": {"value": cpu_cells / cpu_dt / 1e9, "unit": "GCUPS", "cores": O.num_threads(), "kind": "port",
                         "sample": f"first {n_cpu} regions of the stream ({cpu_cells:.3e} cells, {sub.n_pairs} pairs)",
                         "host": f"{platform.machine()} x{os.cpu_count()}"},
        "accuracy_vs_fp64_oracle": {"sample_pairs": int(sub.n_pairs), "max_abs_dlog10": float(d.max()),
                                    "median_abs_dlog10": float(np.median(d)),
                                    "sample": f"first {n_cpu} regions of the stream"},
        "accuracy_vs_fp64_oracle_high_depth_tail": tail,
        "peaks_measured": peaks,
    }
    print(json.dumps(line), flush=True)
    q.close()
    eng.close()
    return 0


def run_calib(args):
    """--calib: workload 3 (4,096 read x haplotype pairs around short tandem repeats).  Times the FP32
    forward and the forward + hand-written backward (ghmm_calib_*, through the torch.autograd.Function) and
    checks the gradient of sum log10 L with respect to the 8 x 20 x 2 (period, repeat) table against FP64
    central differences (step 1e-4, FP64 forward on the GPU) and against the FP64 oracle's adjoint."""
    import numpy as np
    import torch

    from gatk_gb300 import calibration as C, workload as W
    from gatk_gb300.pairhmm import Engine
    from oracle import oracle as O

    eng = Engine()
    wl = W.generate(3)
    cs = C.CalibrationSet(wl)
    cells = int(cs.cells)
    theta = C.default_theta().to(cs.device)

    def timed(fn, reps):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(reps):
            fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / reps

    def fwd():
        with torch.no_grad():
            C.log10_likelihoods(theta, cs, eng, precision=0)

    def fwd_bwd():
        t = theta.detach().requires_grad_(True)
        C.log10_likelihoods(t, cs, eng, precision=0).sum().backward()

    reps = max(args.steps, 10)
    dt_f = timed(fwd, reps)
    clocks = ClockSampler(0)
    clocks.start()
    dt_fb = timed(fwd_bwd, reps)
    clk = clocks.stop()

    # e2e: the parameter table from pinned host memory to the device, forward + backward, its gradient back
    theta_host = theta.detach().cpu().pin_memory()
    grad_host = torch.empty_like(theta_host).pin_memory()

    def fwd_bwd_host():
        t = theta_host.to(cs.device, non_blocking=True).requires_grad_(True)
        C.log10_likelihoods(t, cs, eng, precision=0).sum().backward()
        grad_host.copy_(t.grad, non_blocking=True)

    dt_e2e = timed(fwd_bwd_host, reps)
    # gradient checks
    t = theta.detach().requires_grad_(True)
    C.log10_likelihoods(t, cs, eng, precision=0).sum().backward()
    grad = t.grad.detach().cpu().numpy().reshape(-1, 2)
    used = np.bincount(cs.param_index_np[cs.param_index_np >= 0], minlength=160)
    order = np.nonzero(used)[0]  # every entry some read position uses
    unused_nonzero = int((grad[used == 0] != 0).sum())  # must be 0: unused entries get no gradient
    h = 1e-4
    scale = np.abs(grad).max()
    fd_rel = 0.0
    t_fd = time.perf_counter()
    with torch.no_grad():
        for k in order:
            for comp in (0, 1):
                tp, tm = theta.clone(), theta.clone()
                tp.view(-1, 2)[k, comp] += h
                tm.view(-1, 2)[k, comp] -= h
                sp = float(C.log10_likelihoods(tp, cs, eng, precision=1).sum())
                sm = float(C.log10_likelihoods(tm, cs, eng, precision=1).sum())
                step = float(tp.view(-1, 2)[k, comp].double() - tm.view(-1, 2)[k, comp].double())
                fd = (sp - sm) / step
                fd_rel = max(fd_rel, abs(grad[k, comp] - fd) / max(abs(fd), 1e-2 * scale))
    fd_s = time.perf_counter() - t_fd
    # per-position gradients against the FP64 oracle's adjoint on every pair
    g, c = cs.position_params(theta)
    g = g.detach().requires_grad_(True)
    c = c.detach().requires_grad_(True)
    fn = C._function() if C._FN is None else C._FN
    fn.apply(g, c, cs, eng, 0).sum().backward()
    gg, gc = g.grad.cpu().numpy(), c.grad.cpu().numpy()
    gn, cn = g.detach().cpu().numpy(), c.detach().cpu().numpy()
    pr, ph = wl.pair_index()
    oracle_rel = 0.0
    oracle_cells = 0
    t_or = time.perf_counter()
    for p in range(cs.n_pairs):
        r, hh = int(pr[p]), int(ph[p])
        a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
        _, dg, dc = O.cont_grad(wl.hap(hh), wl.bases[a:b], wl.quals[a:b], gn[a:b].astype(np.float64),
                                cn[a:b].astype(np.float64))
        oracle_cells += (b - a) * len(wl.hap(hh))
        sc = max(np.abs(dg).max(), np.abs(dc).max())
        oracle_rel = max(oracle_rel, np.abs(gg[a:b] - dg).max() / sc, np.abs(gc[a:b] - dc).max() / sc)
    cpu_dt = time.perf_counter() - t_or
    peaks = eng.measure_peaks()
    peak32 = max(peaks["fp32_tflops"], peaks["fp32x2_tflops"])
    line = {
        "metric": "PairHMM calibration: FP32 forward + hand-written backward, GCUPS", "value": cells / dt_fb / 1e9,
        "unit": "GCUPS", "n_gpus": 1, "steps": reps, "warmup": args.warmup, "ms_per_step": dt_fb * 1e3,
        "higher_is_better": True, "dtype": "f32", "data": "synthetic (workload 3: STR regions, seed 3)",
        "config": {"workload": "workload 3: 4,096 read x haplotype pairs, 150 bp reads, 300 bp STR haplotypes",
                   "pairs": cs.n_pairs, "cells": cells, "parameters": "8 x 20 x 2 (period, repeat) log10 table"},
        "forward_gcups": cells / dt_f / 1e9, "forward_ms": dt_f * 1e3,
        "gradient_vs_fp64_central_differences": {"max_rel": float(fd_rel), "params": int(len(order) * 2), "step": h,
                                                 "budget": 1e-3, "used_entries": int(len(order)),
                                                 "unused_entries": int((used == 0).sum()),
                                                 "unused_entries_with_nonzero_gradient": unused_nonzero,
                                                 "seconds": fd_s,
                                                 "relative_to": "max(|fd|, 1e-2 x the largest gradient component)"},
        "gradient_vs_fp64_oracle_adjoint": {"max_rel": float(oracle_rel), "sample_pairs": int(cs.n_pairs)},
        "roofline": {"bound": "fp32_fma_pipe", "achieved": CALIB_FLOP_PER_CELL * cells / dt_fb / 1e12,
                     "peak": peak32, "unit": "TFLOP/s", "frac": CALIB_FLOP_PER_CELL * cells / dt_fb / 1e12 / peak32,
                     "flop_per_cell": CALIB_FLOP_PER_CELL,
                     "kernel": "calib_kernel<float, K, true> over the whole autograd step (latency-bound at 4,096 pairs)"},
        "e2e": {"value": cells / dt_e2e / 1e9, "unit": "GCUPS", "ms_per_step": dt_e2e * 1e3,
                "h2d_bytes_per_step": int(theta_host.numel() * 4), "d2h_bytes_per_step": int(grad_host.numel() * 4),
                "api": "calibration.log10_likelihoods(...).sum().backward() with the table from and the gradient to "
                       "pinned host memory"},
        "gpu_launches": reps,
        "clocks": clk,
        "cpu_baseline": {"value": oracle_cells / cpu_dt / 1e9, "unit": "GCUPS", "cores": 1, "kind": "port",
                         "sample": f"every pair ({cs.n_pairs} pairs, {oracle_cells:.3e} cells): "
                                   "FP64 forward + adjoint of oracle/oracle_grad.c, one pair at a time"},
    }
    print(json.dumps(line), flush=True)
    eng.close()
    return 0


def run_pd(args):
    """--pd: the PD-HMM (LoglessPDPairHMM, DRAGEN-GATK mode) over workload 1's regions with synthetic
    partially-determined haplotypes (1-3 undetermined SNPs and 0-2 undetermined deletions per haplotype,
    seeded).  Device-resident GCUPS of the default path (GHMM_MODE_PD_FP32: read-pair tasks in the packed FP32 PD
    kernel, pairs without a task in the general FP32 one, pairs whose sums underflow recomputed by the FP64 one) and
    of the all-FP64 path (GHMM_MODE_PD), e2e through
    ghmm_pd_compute_regions, accuracy and the CPU baseline against the FP64 PD oracle on the leading regions."""
    import numpy as np

    from gatk_gb300 import native, workload as W
    from gatk_gb300.pairhmm import Engine, _read_prep
    from oracle import oracle as O

    eng = Engine()
    peaks = eng.measure_peaks()
    n_regions = args.regions or 1000
    wl = W.generate(1, regions=n_regions)
    pd = W.pd_flags(wl, 5)
    cells = int(wl.cells_per_region().sum())
    batch = eng.pd_batch(wl, pd)

    def timed(mode):
        for _ in range(args.warmup):
            batch.forward(mode)
        sts = []
        for _ in range(args.steps):
            batch.forward(mode)
            sts.append(batch.stats())
        return sts, batch.results()

    clocks = ClockSampler(0)
    clocks.start()
    sts, res = timed(native.MODE_PD_FP32)
    clk = clocks.stop()
    sts64, res64 = timed(native.MODE_PD)
    ms = statistics.mean(s["ms_total"] for s in sts)
    ms_fp32 = statistics.mean(s["ms_fp32"] for s in sts)
    ms_rerun = statistics.mean(s["ms_fp64"] for s in sts)
    ms64 = statistics.mean(s["ms_total"] for s in sts64)
    ms64_kernel = statistics.mean(s["ms_fp64"] for s in sts64)
    n_rerun = int(sts[-1]["n_rerun"])
    io = batch.stats()
    batch.close()
    # e2e: the C-ABI call from host buffers, its region structs built before the timed calls (as the regular e2e)
    L = eng.L
    out = np.empty(max(wl.n_pairs, 1), dtype=np.float64)
    regs = W.as_pd_regions(wl, pd)

    def e2e_call():
        native.check(L.ghmm_pd_compute_regions(eng.handle, regs, wl.n_regions, out.ctypes.data_as(native._f64p)),
                     eng.handle)

    # the DRAGEN-GATK chain from raw reads: DRAGstr imputation on the device, then the PD-HMM, in one call
    mapq = np.random.default_rng(31).integers(20, 70, size=wl.n_reads)
    regs_raw = W.as_pd_raw_regions(wl, pd, mapq, True)
    prep = _read_prep(18, True, 3.0, 10, _prep_tables(), wl)
    out_raw = np.empty(max(wl.n_pairs, 1), dtype=np.float64)

    def raw_call():
        native.check(L.ghmm_pd_compute_regions_raw(eng.handle, regs_raw, wl.n_regions, ctypes.byref(prep),
                                                   out_raw.ctypes.data_as(native._f64p)), eng.handle)

    def timed_calls(fn):
        for _ in range(max(1, min(args.warmup, 2))):
            fn()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            fn()
        return (time.perf_counter() - t0) / args.steps

    dt_e2e = timed_calls(e2e_call)
    dt_raw = timed_calls(raw_call)
    out = out[: wl.n_pairs]
    n_cpu, cpu_cells = cpu_sample(wl, args.cpu_cells / 4)
    sub = wl.subset(0, n_cpu)
    sub_pd = pd[: int(wl.hap_off[int(wl.region_hap_off[n_cpu])])]
    t1 = time.perf_counter()
    ref = O.pd_compute_workload(sub, sub_pd)
    cpu_dt = time.perf_counter() - t1
    d = absdiff(res[: sub.n_pairs], ref)
    d64 = absdiff(res64[: sub.n_pairs], ref)
    dall = absdiff(res[: wl.n_pairs], res64[: wl.n_pairs])
    flop_per_cell = 11  # M: mul + 2 fma, D: mul + fma, I: mul + fma (FMA = 2), as the regular recurrence
    achieved = flop_per_cell * cells / (ms_fp32 * 1e-3) / 1e12
    peak32 = max(peaks["fp32_tflops"], peaks["fp32x2_tflops"])
    dp_achieved = 11 * cells / (ms64_kernel * 1e-3) / 1e12
    line = {
        "metric": "PD-HMM GCUPS (partially determined haplotypes) on 1 GB300", "value": cells / (ms * 1e-3) / 1e9,
        "unit": "GCUPS", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "dtype": "f32",
        "data": "synthetic (workload 1 regions with seeded PD flags)",
        "config": {"workload": f"first {n_regions} regions of workload 1 with 1-3 undetermined SNPs and 0-2 undetermined "
                               "deletions per haplotype", "regions": n_regions, "pairs": wl.n_pairs, "cells": cells,
                   "mode": "GHMM_MODE_PD_FP32 (FP32 PD kernels, FP64 reruns of underflows)"},
        "roofline": {"bound": "fp32_fma_pipe", "achieved": achieved, "peak": peak32, "unit": "TFLOP/s",
                     "frac": achieved / peak32, "flop_per_cell": flop_per_cell,
                     "kernel": "pd_bucket_kernel<K> (read-pair tasks) and pd_kernel<float, K> (pairs without a task): the FP32 pass",
                     "ms_fp32_pass": ms_fp32,
                     "ms_fp64_reruns": ms_rerun},
        "fp64_rerun": {"pairs": n_rerun, "fraction": n_rerun / max(1, wl.n_pairs)},
        "fp64_mode": {"value": cells / (ms64 * 1e-3) / 1e9, "unit": "GCUPS", "ms_per_step": ms64,
                      "mode": "GHMM_MODE_PD (every pair in FP64 at the reference's 2^1020 scale)",
                      "roofline": {"bound": "fp64_pipe", "achieved": dp_achieved, "peak": peaks["fp64_tflops"],
                                   "unit": "TFLOP/s", "frac": dp_achieved / peaks["fp64_tflops"]},
                      "max_abs_dlog10_vs_oracle": float(d64.max())},
        "e2e": {"value": cells / dt_e2e / 1e9, "unit": "GCUPS", "ms_per_step": dt_e2e * 1e3,
                "h2d_bytes_per_step": int(io["h2d_bytes"]), "d2h_bytes_per_step": int(io["d2h_bytes"]),
                "steps": args.steps, "api": "ghmm_pd_compute_regions", "matches_batch": bool(np.array_equal(out, res))},
        "e2e_raw_dragstr": {"value": cells / dt_raw / 1e9, "unit": "GCUPS", "ms_per_step": dt_raw * 1e3,
                            "steps": args.steps,
                            "api": "ghmm_pd_compute_regions_raw with the reference's example DRAGstr model "
                                   "(imputation on the device, then the PD-HMM; seeded MAPQ 20-69)"},
        "gpu_launches": int(sts[-1]["n_launches"]) * args.steps,
        "clocks": clk,
        "cpu_baseline": {"value": cpu_cells / cpu_dt / 1e9, "unit": "GCUPS", "cores": O.num_threads(), "kind": "port",
                         "sample": f"first {n_cpu} regions ({cpu_cells:.3e} cells, {sub.n_pairs} pairs)",
                         "host": f"{platform.machine()} x{os.cpu_count()}"},
        "accuracy_vs_fp64_oracle": {"sample_pairs": int(sub.n_pairs), "max_abs_dlog10": float(d.max()),
                                    "median_abs_dlog10": float(np.median(d))},
        # every pair of the timed workload: the default FP32 path against the GPU's all-FP64 mode (itself pinned to the
        # oracle on the sample above, fp64_mode.max_abs_dlog10_vs_oracle)
        "accuracy_vs_gpu_fp64_full_workload": {"pairs": int(len(dall)), "max_abs_dlog10": float(dall.max()),
                                               "median_abs_dlog10": float(np.median(dall)),
                                               "pairs_above_1e-3": int((dall > 1e-3).sum())},
    }
    print(json.dumps(line), flush=True)
    eng.close()
    return 0


def _prep_tables():
    """The DRAGstr model the reference's HaplotypeCaller integration tests run with (its example parameter file,
    extracted to tests/golden/dragstr_cases.json): GOP and GCP tables of 8 periods x 20 repeat lengths."""
    import numpy as np

    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "tests", "golden", "dragstr_cases.json")) as f:
        t = json.load(f)["example_params"]
    return np.array(t["gop"]), np.array(t["gcp"])


def measured_hbm_peak() -> float:
    """HBM copy bandwidth in GB/s from MEASURED_PEAKS.json (6800 GB/s, an earlier GB300 measurement, without it)."""
    try:
        with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "MEASURED_PEAKS.json")) as f:
            return float(json.load(f)["hbm_gbs"])
    except (OSError, KeyError, ValueError):
        return 6800.0


def _oracle_prepared(wl, mapq, raw_kw):
    """wl with its quality planes replaced by oracle/readprep.py's preparation of its raw reads."""
    import numpy as np

    from gatk_gb300 import workload as W
    from oracle import readprep as RP

    planes = [np.empty_like(wl.bases) for _ in range(4)]
    for r in range(wl.n_reads):
        a, e = int(wl.read_off[r]), int(wl.read_off[r + 1])
        _, q, i, d, g = RP.prepare_read(wl.bases[a:e], wl.quals[a:e], wl.ins[a:e], wl.dels[a:e], int(mapq[r]),
                                        rate_factor=raw_kw.get("pcr_rate_factor", 3.0), dragstr=raw_kw.get("dragstr"))
        for k, v in enumerate((q, i, d, g)):
            planes[k][a:e] = np.frombuffer(v, dtype=np.uint8)
    return W.Workload(region_read_off=wl.region_read_off, region_hap_off=wl.region_hap_off, read_off=wl.read_off,
                      bases=wl.bases, quals=planes[0], ins=planes[1], dels=planes[2], gcp=planes[3],
                      hap_off=wl.hap_off, hap_bases=wl.hap_bases, out_off=wl.out_off)


PREP_BYTES_PER_BASE = {"pcr": 7, "dragstr": 6}  # pcr: read bases, quals, BI, BD; write quals, BI, BD.
#                                                 dragstr: read bases, quals; write quals, GOP (ins = del), GCP


def run_prep(args):
    """--prep: the read preparation before the PairHMM on the device (ghmm_batch_create_raw), over every read of
    workload 1 with seeded raw base qualities, BI / BD tags and mapping qualities.  Two imputations:
    `pcr` (PairHMMLikelihoodCalculationEngine.modifyReadQualities with the CONSERVATIVE PCR indel model and the
    standard imputation) and `dragstr` (DragstrPairHMMInputScoreImputator with the reference's example DRAGstr
    model).  `value` is reads prepared per second by the device kernels (CUDA events around them, planes resident);
    e2e is the likelihood call ghmm_compute_regions_raw from raw reads in host memory against the same call on
    planes prepared beforehand (ghmm_compute_regions): the difference is what preparation costs inside a call.
    The CPU baseline is the C restatement (oracle/readprep_oracle.c) over every read on all host cores, whose planes
    must all equal the device's."""
    import numpy as np

    from gatk_gb300 import native, workload as W
    from gatk_gb300.pairhmm import Engine
    from oracle import readprep as RP

    mode = args.prep
    eng = Engine()
    n_regions = args.regions or 0
    wl = W.generate(1, regions=n_regions) if n_regions else W.generate(1)
    rng = np.random.default_rng(23)
    wl.quals[:] = rng.integers(2, 45, size=len(wl.quals)).astype(np.uint8)
    wl.ins[:] = rng.integers(20, 50, size=len(wl.ins)).astype(np.uint8)
    wl.dels[:] = rng.integers(20, 50, size=len(wl.dels)).astype(np.uint8)
    mapq = rng.integers(10, 70, size=wl.n_reads)
    kw = {"pcr_rate_factor": 3.0}
    if mode == "dragstr":
        kw["dragstr"] = _prep_tables()
    bases = int(len(wl.bases))
    cells = int(wl.cells_per_region().sum())
    for _ in range(args.warmup):
        with eng.raw_batch(wl, mapq, **kw) as b:
            b.stats()
    clocks = ClockSampler(0)
    clocks.start()
    ms = []
    for _ in range(args.steps):
        with eng.raw_batch(wl, mapq, **kw) as b:
            ms.append(b.stats()["ms_prep"])
    clk = clocks.stop()
    with eng.raw_batch(wl, mapq, **kw) as b:
        planes = b.read_planes()
        b.forward()
        fst = b.stats()
    ms_prep = statistics.mean(ms)
    # e2e: raw reads in host memory -> likelihoods in host memory, against the call on prepared planes
    prepared = W.Workload(region_read_off=wl.region_read_off, region_hap_off=wl.region_hap_off, read_off=wl.read_off,
                          bases=wl.bases, quals=planes[1], ins=planes[2], dels=planes[3], gcp=planes[4],
                          hap_off=wl.hap_off, hap_bases=wl.hap_bases, out_off=wl.out_off)
    # the per-read struct arrays are built once, outside the timed calls, as a JNI caller passes its arrays
    from gatk_gb300.pairhmm import _read_prep

    regs_raw = W.as_raw_regions(wl, mapq, True)
    rp = _read_prep(18, True, 3.0, 10, kw.get("dragstr"), wl)
    regs_prep = prepared.as_regions()
    raw_out = np.empty(wl.n_pairs, dtype=np.float64)
    prep_out = np.empty(wl.n_pairs, dtype=np.float64)
    L, h = eng.L, eng.handle

    def call_raw():
        native.check(L.ghmm_compute_regions_raw(h, regs_raw, wl.n_regions, ctypes.byref(rp),
                                                raw_out.ctypes.data_as(native._f64p)), h)

    def call_prepared():
        native.check(L.ghmm_compute_regions(h, regs_prep, wl.n_regions, prep_out.ctypes.data_as(native._f64p)), h)

    call_raw()
    call_prepared()
    t_raw, t_prep = [], []
    for _ in range(max(1, min(args.steps, 3))):
        t0 = time.perf_counter()
        call_raw()
        t_raw.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        call_prepared()
        t_prep.append(time.perf_counter() - t0)
    dt_raw, dt_prep = min(t_raw), min(t_prep)
    # CPU baseline and parity: the C restatement (oracle/readprep_oracle.c) over every read on all host cores
    from oracle import oracle as O

    t1 = time.perf_counter()
    want = O.prepare_reads(wl.read_off, wl.bases, wl.quals, wl.ins, wl.dels, mapq, rate_factor=3.0,
                           dragstr=kw.get("dragstr"))
    cpu_dt = time.perf_counter() - t1
    diff = np.zeros(len(wl.bases), dtype=bool)
    for k in range(4):
        diff |= planes[k + 1] != want[k]
    bad_reads = np.unique(np.searchsorted(wl.read_off, np.nonzero(diff)[0], side="right") - 1)
    n_cpu, mism = wl.n_reads, int(len(bad_reads))
    # the Python restatement, for the record, on the leading reads for a bounded time
    n_py = 0
    t2 = time.perf_counter()
    while n_py < wl.n_reads and time.perf_counter() - t2 < args.cpu_seconds:
        a, e = int(wl.read_off[n_py]), int(wl.read_off[n_py + 1])
        RP.prepare_read(wl.bases[a:e], wl.quals[a:e], wl.ins[a:e], wl.dels[a:e], int(mapq[n_py]), rate_factor=3.0,
                        dragstr=kw.get("dragstr"))
        n_py += 1
    py_rate = n_py / (time.perf_counter() - t2)
    algo_bytes = PREP_BYTES_PER_BASE[mode] * bases
    achieved = algo_bytes / (ms_prep * 1e-3) / 1e9
    peak = measured_hbm_peak()
    line = {
        "metric": f"reads prepared per second ({mode} imputation) on 1 GB300", "value": wl.n_reads / (ms_prep * 1e-3),
        "unit": "reads/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_prep,
        "higher_is_better": True, "dtype": "u8", "data": "synthetic (workload 1 reads with seeded raw qualities)",
        "config": {"workload": f"every read of workload 1 ({wl.n_regions} regions, {wl.n_reads} reads, {bases} bases), "
                               f"{mode} imputation" + (" with the reference's example DRAGstr model (8 x 20)"
                                                       if mode == "dragstr" else ", CONSERVATIVE PCR model"),
                   "reads": wl.n_reads, "bases": bases},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "bytes_per_base": PREP_BYTES_PER_BASE[mode],
                     "kernel": "prep_kernel + dragstr_kernel" if mode == "dragstr" else "prep_kernel"},
        "e2e": {"value": cells / dt_raw / 1e9, "unit": "GCUPS", "ms_per_step": dt_raw * 1e3,
                "api": "ghmm_compute_regions_raw (per-read pointer arrays built before the timed calls)",
                "prepared_planes_api": "ghmm_compute_regions", "prepared_planes_ms": dt_prep * 1e3,
                "prepared_planes_gcups": cells / dt_prep / 1e9,
                "h2d_bytes_per_step": int(5 * bases + len(wl.hap_bases) + 4 * wl.n_reads),
                "d2h_bytes_per_step": int(8 * wl.n_pairs),
                "max_abs_dlog10_vs_prepared_planes": float(absdiff(raw_out, prep_out).max()),
                "fp64_direct_pairs": int(fst["n_fp64_direct"]), "fp64_rerun_pairs": int(fst["n_rerun"])},
        "gpu_launches": args.steps * (2 if mode == "dragstr" else 1),
        "clocks": clk,
        "cpu_baseline": {"value": n_cpu / cpu_dt, "unit": "reads/s", "cores": O.num_threads(), "kind": "port",
                         "sample": f"all {n_cpu} reads through oracle/readprep_oracle.c (C, OpenMP over reads)",
                         "python_restatement_reads_per_s": py_rate,
                         "host": f"{platform.machine()} x{os.cpu_count()}"},
        "parity": {"reads": n_cpu, "mismatched_reads": mism},
    }
    print(json.dumps(line), flush=True)
    eng.close()
    return 0


# calibration step: forward (11), checkpointed recompute (11) and the adjoint wavefront (about twice a forward, 22)
CALIB_FLOP_PER_CELL = 44

SW_OPS_PER_CELL = 12  # calculateMatrix's inner loop: 5 adds, 6 compares / maxima, the base compare


def run_sw(args):
    """--sw: the step after the likelihoods, AssemblyBasedCallerUtils.realignReadsToTheirBestHaplotype on workload
    1: every read realigned with Smith-Waterman (ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS, SOFTCLIP, the exact-
    substring shortcut) against the haplotype its likelihoods favour, ties broken toward the region's first
    (reference) haplotype.  A step is one ghmm_batch_realign over every read of the workload with the sequences and
    the PairHMM likelihoods resident on the GPU (cigars come back to the host inside the step).  `value` is GCUPS
    over the cells of the alignments that ran the score recurrence, per device second; `e2e` is the same alignments
    through ghmm_sw_align_batch from host buffers (marshal, H2D, kernels, D2H).  The CPU baseline is the C
    restatement of SmithWatermanJavaAligner on every host core over the leading reads; its cigars and offsets must
    equal the GPU's."""
    import ctypes

    import numpy as np

    from gatk_gb300 import native, workload as W
    from gatk_gb300 import smithwaterman as SWG
    from gatk_gb300.pairhmm import Batch, Engine
    from oracle import oracle as O

    eng = Engine()
    wl = W.generate(args.workload, regions=args.regions or (100 if args.workload == 2 else None))
    n_regions = wl.n_regions
    batch = Batch(eng, wl)
    batch.forward()
    prio = np.zeros(wl.n_haps, dtype=np.float64)
    prio[wl.region_hap_off[:-1]] = 1.0  # HAPLOTYPE_ALIGNMENT_TIEBREAKING_PRIORITY: reference haplotype, no cigars
    for _ in range(args.warmup):
        best, inf, res = SWG.realign_batch(batch, prio)
    clocks = ClockSampler(0)
    clocks.start()
    sts = []
    t0 = time.perf_counter()
    for _ in range(args.steps):
        best, inf, res = SWG.realign_batch(batch, prio)
        sts.append(SWG.sw_stats(eng.L, eng.handle))
    dt_call = (time.perf_counter() - t0) / args.steps
    clk = clocks.stop()
    st = sts[-1]
    cells = st["cells"]
    ms_dev = statistics.mean(x["ms_device"] for x in sts)
    ms_fwd = statistics.mean(x["ms_forward"] for x in sts)
    batch.close()
    # the same (haplotype, read) pairs from host buffers through the batched C-ABI call
    pairs = np.zeros(wl.n_reads, dtype=[("ref", "<u8"), ("alt", "<u8"), ("ref_len", "<i4"), ("alt_len", "<i4")])
    region_of = np.repeat(np.arange(wl.n_regions), np.diff(wl.region_read_off))
    hap = wl.region_hap_off[region_of] + best
    pairs["ref"] = wl.hap_bases.ctypes.data + wl.hap_off[hap]
    pairs["ref_len"] = wl.hap_off[hap + 1] - wl.hap_off[hap]
    pairs["alt"] = wl.bases.ctypes.data + wl.read_off[:-1]
    pairs["alt_len"] = np.diff(wl.read_off)
    cap = int(2 * pairs["alt_len"].sum() + 4 * wl.n_reads)
    res2, off2, start2, len2, ops2 = SWG._result(wl.n_reads, cap)
    p = SWG.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS.as_native()
    pp = ctypes.cast(pairs.ctypes.data, ctypes.POINTER(native.SwPair))
    for _ in range(2):
        native.check(eng.L.ghmm_sw_align_batch(eng.handle, pp, wl.n_reads, ctypes.byref(p), native.SW_SOFTCLIP,
                                               native.SW_SUBSTRING_SHORTCUT, ctypes.byref(res2)), eng.handle)
    t0 = time.perf_counter()
    native.check(eng.L.ghmm_sw_align_batch(eng.handle, pp, wl.n_reads, ctypes.byref(p), native.SW_SOFTCLIP,
                                           native.SW_SUBSTRING_SHORTCUT, ctypes.byref(res2)), eng.handle)
    dt_e2e = time.perf_counter() - t0
    st2 = SWG.sw_stats(eng.L, eng.handle)
    same = (np.array_equal(off2[:wl.n_reads], res.offset) and np.array_equal(len2[:wl.n_reads], res.cigar_len)
            and np.array_equal(ops2[:res2.cigar_total], res.cigar_ops))
    # CPU baseline and parity on the leading reads
    lens = pairs["ref_len"].astype(np.int64) * pairs["alt_len"]
    n_cpu = int(min(wl.n_reads, np.searchsorted(np.cumsum(lens), args.cpu_cells / 2) + 1))
    t1 = time.perf_counter()
    ops_c, start_c, n_c, off_c = O.sw_align_pairs(wl.hap_bases, wl.hap_off[hap[:n_cpu]], pairs["ref_len"][:n_cpu],
                                                  wl.bases, wl.read_off[:n_cpu], pairs["alt_len"][:n_cpu],
                                                  (10, -15, -30, -5), native.SW_SOFTCLIP, True)
    cpu_dt = time.perf_counter() - t1
    mism = 0
    for i in range(n_cpu):
        if off_c[i] != res.offset[i] or not np.array_equal(ops_c[start_c[i]:start_c[i] + n_c[i]], res.ops(i)):
            mism += 1
    with SWG.SmithWatermanCudaAligner() as a:
        peak = a.measure_peak()
    achieved = SW_OPS_PER_CELL * cells / (ms_fwd * 1e-3) / 1e12
    line = {
        "metric": "Smith-Waterman realignment GCUPS (reads to their best haplotype) on 1 GB300",
        "value": cells / (ms_dev * 1e-3) / 1e9, "unit": "GCUPS", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_dev, "higher_is_better": True, "dtype": "int32",
        "data": f"synthetic (workload {args.workload}; best haplotypes from the PairHMM forward)",
        "config": {"workload": f"config{args.workload}: {n_regions} regions, every read against its best haplotype",
                   "reads": int(wl.n_reads), "alignments_with_recurrence": int(st["n_alignments"] - st["n_shortcut"]),
                   "substring_shortcut": int(st["n_shortcut"]), "cells": int(cells), "chunks": int(st["chunks"]),
                   "int16_paired_alignments": int(st["n_int16"]),
                   "parameters": "ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS (10, -15, -30, -5), SOFTCLIP"},
        "realign_call_ms": dt_call * 1e3,
        "realign_host_ms": statistics.mean(x["ms_host"] for x in sts),
        "alignments_per_s": wl.n_reads / (dt_call),
        "roofline": {"bound": "int32_alu", "achieved": achieved, "peak": peak, "unit": "Tops/s",
                     "frac": achieved / peak, "ops_per_cell": SW_OPS_PER_CELL, "kernel": "sw_forward_kernel<K>",
                     "ms_forward": ms_fwd, "peak_source": "measured in this run: max.s32 register loop over all SMs"},
        "e2e": {"value": st2["cells"] / dt_e2e / 1e9, "unit": "GCUPS", "ms_per_step": dt_e2e * 1e3,
                "h2d_bytes_per_step": int(st2["h2d_bytes"]), "d2h_bytes_per_step": int(st2["d2h_bytes"]),
                "api": "ghmm_sw_align_batch (host pairs, SOFTCLIP, substring shortcut)", "matches_realign": bool(same),
                "host_ms": st2["ms_host"], "device_ms": st2["ms_device"]},
        "gpu_launches": int(st["launches"]),
        "clocks": clk,
        "cpu_baseline": {"value": float(lens[:n_cpu].sum()) / cpu_dt / 1e9, "unit": "GCUPS", "cores": os.cpu_count(),
                         "kind": "port", "sample": f"first {n_cpu} reads against their best haplotypes "
                                                   f"({float(lens[:n_cpu].sum()):.3e} cells)",
                         "host": f"{platform.machine()} x{os.cpu_count()}"},
        "parity_vs_oracle": {"sample_reads": n_cpu, "mismatches": mism},
    }
    print(json.dumps(line), flush=True)
    eng.close()
    return 0 if mism == 0 and same else 1


def apply_tuning(args, eng, wl):
    """--tuning K,KM,C sets the launch shape; --autotune runs the native autotuner on the whole workload
    (untimed) over the candidates it names.  Returns what was used."""
    if args.autotune:
        cands = [tuple(int(x) for x in c.split(",")) for c in args.autotune.split(";")]
        t = eng.autotune(wl, candidates=cands, use_cache=False, sample_cells=float("inf"))
        return {"max_rows_per_lane": t["max_rows_per_lane"], "max_rows_per_lane_multi": t["max_rows_per_lane_multi"],
                "chunk_cols": t["chunk_cols"], "autotune_ms": t["ms"], "autotune_s": t["search_s"]}
    if args.tuning:
        k, km, c = (int(x) for x in args.tuning.split(","))
        eng.set_tuning(k, km, c)
    k, km, c = eng.get_tuning()
    return {"max_rows_per_lane": k, "max_rows_per_lane_multi": km, "chunk_cols": c}


def absdiff(got, ref):
    """|got - ref|, where equal infinities count as 0: a pair whose likelihood underflows even the FP64
    2^1020 scale is -Infinity in LoglessPairHMM too."""
    import numpy as np

    got, ref = np.asarray(got), np.asarray(ref)
    same_inf = np.isinf(got) & np.isinf(ref) & (got == ref)
    with np.errstate(invalid="ignore"):
        return np.where(same_inf, 0.0, np.abs(got - ref))


def ctypes_addr(ptr) -> int:
    import ctypes

    return ctypes.cast(ptr, ctypes.c_void_p).value


def read_profile_traffic():
    """DRAM bytes per launch set of the FP32 kernels from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "fp32_bucket_kernel_workload1.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("traffic_bytes_per_launch_set:"):
                    return float(line.split(":", 1)[1].strip())
    except OSError:
        pass
    return None


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", type=int, default=1)
    ap.add_argument("--regions", type=int, default=0, help="regions per rank, or in all with --scaling strong "
                    "(0: the workload's full size)")
    ap.add_argument("--scaling", choices=["weak", "strong"], default="weak",
                    help="weak: every rank runs its own full-size block of regions; strong: the ranks split one "
                         "workload with the library's split (ghmm_multi_plan)")
    ap.add_argument("--cpu-cells", type=float, default=CPU_SAMPLE_CELLS)
    ap.add_argument("--plain-cells", type=float, default=PLAIN_SAMPLE_CELLS)
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-full-check", action="store_true",
                    help="skip the comparison of every timed result with the GPU's FP64 mode")
    ap.add_argument("--stream", action="store_true",
                    help="push the workload one region at a time through the queue (default workload 4)")
    ap.add_argument("--batch-cells", type=float, default=2e11, help="queue batch size in cells (--stream)")
    ap.add_argument("--tuning", default="", help="launch shape K,KM,CHUNK_COLS (rows per lane, multi-strip rows "
                    "per lane, haplotype columns per task)")
    ap.add_argument("--autotune", default="", help="autotune over candidates 'K,KM,C;K,KM,C;...' on the whole "
                    "workload before timing")
    ap.add_argument("--pd", action="store_true", help="PD-HMM over workload 1 regions with synthetic PD flags")
    ap.add_argument("--calib", action="store_true",
                    help="time the calibration forward + backward on workload 3 and check its gradient")
    ap.add_argument("--prep", choices=["pcr", "dragstr"], default=None,
                    help="read preparation on the device over every workload 1 read (PCR model or DRAGstr)")
    ap.add_argument("--cpu-seconds", type=float, default=3.0,
                    help="time bound of the --prep Python-restatement sample (the C baseline covers every read)")
    ap.add_argument("--raw", choices=["pcr", "dragstr"], default=None,
                    help="with --stream: push raw reads (ghmm_queue_push_raw), prepared on the device")
    ap.add_argument("--sw", action="store_true",
                    help="Smith-Waterman realignment of every workload 1 read to its best haplotype")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.stream and "--workload" not in " ".join(sys.argv):
        args.workload = 4
    if args.impl == "reference":
        return run_reference(args)
    if args.stream:
        return run_stream(args)
    if args.calib:
        return run_calib(args)
    if args.pd:
        return run_pd(args)
    if args.sw:
        return run_sw(args)
    if args.prep:
        return run_prep(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
