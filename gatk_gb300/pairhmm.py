"""Host-side mirror of GATK's PairHMM plugin interface for the CUDA_LOGLESS implementation.

Reference interface (paths inside the GATK repository):
  PairHMM.Implementation, makeNewHMM(PairHMMNativeArguments)   utils/pairhmm/PairHMM.java:40-109
  VectorLoglessPairHMM (the JNI-backed implementation this mirrors):
      constructor: load() else HardwareFeatureException         utils/pairhmm/VectorLoglessPairHMM.java:57-82
      initialize(haplotypes, perSampleReadList, maxR, maxH)     :89-102
      computeLog10Likelihoods(matrix, processedReads, imputator) :108-159
      close()                                                   :163-168
  PairHMMNativeArguments {maxNumberOfThreads, useDoublePrecision} (HC/PairHMMNativeArgumentCollection.java:11-23)

Every computation goes through libghmm.so on the GPU; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass
from typing import Iterable, Sequence

import numpy as np

from . import native
from .workload import Workload


class HardwareFeatureException(RuntimeError):
    """UserException.HardwareFeatureException: the accelerated implementation is not available."""


@dataclass
class PairHMMNativeArguments:
    max_number_of_threads: int = 0
    use_double_precision: bool = False
    device: int = 0


class Implementation(enum.Enum):
    """The PairHMM.Implementation constant this package adds (CUDA_LOGLESS)."""

    CUDA_LOGLESS = "CUDA_LOGLESS"

    def make_new_hmm(self, args: PairHMMNativeArguments | None = None) -> "CudaLoglessPairHMM":
        return CudaLoglessPairHMM(args)


def _u8(x) -> np.ndarray:
    if isinstance(x, (bytes, bytearray)):
        return np.frombuffer(bytes(x), dtype=np.uint8)
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint8))


def _read_prep(threshold, cap_to_mapq, pcr_rate_factor, gcp, dragstr, keep_with) -> native.ReadPrep:
    """ghmm_read_prep; dragstr = (gop, gcp) tables [max_period][max_repeats] (DragstrParams) or None.  The tables are
    kept alive on keep_with (a Workload, or a list) for as long as the library may read them."""
    d = None
    if dragstr is not None:
        gop_t = np.ascontiguousarray(dragstr[0], dtype=np.float64)
        gcp_t = np.ascontiguousarray(dragstr[1], dtype=np.float64)
        if gop_t.ndim != 2 or gop_t.shape != gcp_t.shape:
            raise ValueError("DRAGstr gop and gcp tables must both be [max_period][max_repeats]")
        d = native.Dragstr(gop_t.shape[0], gop_t.shape[1], gop_t.ctypes.data, gcp_t.ctypes.data)
        (keep_with if isinstance(keep_with, list) else keep_with._keep).append((gop_t, gcp_t, d))
    return native.ReadPrep(int(threshold), int(cap_to_mapq), float(pcr_rate_factor), int(gcp), 0,
                           ctypes.addressof(d) if d is not None else None)


class _Context:
    def __init__(self, args: PairHMMNativeArguments):
        L = native.lib()
        if not L.ghmm_load():
            raise HardwareFeatureException("Machine does not support the CUDA PairHMM (no compute capability 10.3 GPU).")
        a = native.Args(args.device, args.max_number_of_threads, int(args.use_double_precision), 0)
        h = ctypes.c_void_p()
        rc = L.ghmm_initialize(ctypes.byref(a), ctypes.byref(h))
        if rc == native.GHMM_ERR_UNSUPPORTED:
            raise HardwareFeatureException(native.last_error(None))
        native.check(rc, None)
        self.h = h
        self.L = L

    def close(self):
        if self.h:
            self.L.ghmm_done(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@dataclass(frozen=True)
class StandardPairHMMInputScoreImputator:
    """StandardPairHMMInputScoreImputator.newInstance(gcp): insertion / deletion GOP from the read's BI / BD tags (45
    without them), a constant gap continuation penalty (HC/StandardPairHMMInputScoreImputator.java:55-74)."""
    gcp: int = 10


@dataclass(frozen=True)
class DragstrPairHMMInputScoreImputator:
    """DragstrPairHMMInputScoreImputator.of(DragstrParams): GOP and GCP tables [period - 1][repeats - 1]
    (HC/DragstrPairHMMInputScoreImputator.java:45-88)."""
    gop: np.ndarray
    gcp: np.ndarray


class CudaLoglessPairHMM:
    """PairHMM backed by the GB300 kernels (VectorLoglessPairHMM's contract).

    ``initialize`` stores the haplotypes; ``compute_log10_likelihoods`` takes the processed reads as
    (bases, quals, insertion GOP, deletion GOP, GCP) tuples and returns the read-major log10
    likelihood array (also kept as ``get_log_likelihood_array()``).
    """

    def __init__(self, args: PairHMMNativeArguments | None = None):
        self.args = args or PairHMMNativeArguments()
        self._ctx = _Context(self.args)
        self._haps: list[np.ndarray] = []
        self._last: np.ndarray | None = None

    # PairHMM.initialize(List<Haplotype>, Map, int, int)
    def initialize(self, haplotypes: Sequence, per_sample_reads=None, read_max_length: int = 0,
                   haplotype_max_length: int = 0) -> None:
        self._haps = [_u8(h) for h in haplotypes]

    # PairHMM.computeLog10Likelihoods(LikelihoodMatrix, List<GATKRead>, PairHMMInputScoreImputator)
    def compute_log10_likelihoods(self, reads: Iterable[Sequence]) -> np.ndarray | None:
        reads = [tuple(_u8(x) for x in r) for r in reads]
        if not reads:  # PairHMM.java:199-201: nothing to do
            return None
        for r in reads:
            if len(r) != 5 or any(len(x) != len(r[0]) for x in r):
                raise ValueError("each read needs bases, quals, ins, del and gcp arrays of equal length")
        nr, nh = len(reads), len(self._haps)
        rs = (native.Read * nr)()
        for i, (b, q, ins, dl, g) in enumerate(reads):
            rs[i] = native.Read(b.ctypes.data_as(native._u8p), q.ctypes.data_as(native._u8p),
                                ins.ctypes.data_as(native._u8p), dl.ctypes.data_as(native._u8p),
                                g.ctypes.data_as(native._u8p), len(b))
        hs = (native.Hap * max(nh, 1))()
        for i, h in enumerate(self._haps):
            hs[i] = native.Hap(h.ctypes.data_as(native._u8p), len(h))
        out = np.empty(nr * nh, dtype=np.float64)
        rc = self._ctx.L.ghmm_compute_likelihoods(self._ctx.h, rs, nr, hs, nh, out.ctypes.data_as(native._f64p))
        if rc == native.GHMM_ERR_ARG:
            raise ValueError(native.last_error(self._ctx.h))
        native.check(rc, self._ctx.h)
        self._last = out
        return out

    def compute_log10_likelihoods_raw(self, reads: Iterable[Sequence], imputator=None, base_quality_threshold: int = 18,
                                      cap_to_mapq: bool = True, pcr_rate_factor: float = 3.0) -> np.ndarray | None:
        """The same step from unprocessed reads, as PairHMMLikelihoodCalculationEngine.computeReadLikelihoods runs it:
        each read is (bases, base qualities, BI tag or None, BD tag or None, mapping quality); modifyReadQualities
        (MAPQ cap, threshold, PCR indel model) and the imputator's penalties are applied on the device
        (ghmm_compute_regions_raw).  imputator: StandardPairHMMInputScoreImputator (default, GCP 10) or
        DragstrPairHMMInputScoreImputator."""
        reads = list(reads)
        if not reads:
            return None
        imputator = imputator or StandardPairHMMInputScoreImputator()
        keep = []
        rr = (native.RawRead * len(reads))()
        for i, (b, q, ins, dl, mq) in enumerate(reads):
            b, q = _u8(b), _u8(q)
            ins = None if ins is None else _u8(ins)
            dl = None if dl is None else _u8(dl)
            if len(q) != len(b) or (ins is not None and len(ins) != len(b)) or (dl is not None and len(dl) != len(b)):
                raise ValueError("each read's quality arrays must match its bases in length")
            keep.append((b, q, ins, dl))
            rr[i] = native.RawRead(b.ctypes.data, q.ctypes.data, ins.ctypes.data if ins is not None else None,
                                   dl.ctypes.data if dl is not None else None, len(b), int(mq))
        nh = len(self._haps)
        hs = (native.Hap * max(nh, 1))()
        for i, h in enumerate(self._haps):
            hs[i] = native.Hap(h.ctypes.data_as(native._u8p), len(h))
        region = native.RawRegion(ctypes.addressof(rr), len(reads), ctypes.addressof(hs), nh)
        if isinstance(imputator, DragstrPairHMMInputScoreImputator):
            prep = _read_prep(base_quality_threshold, cap_to_mapq, pcr_rate_factor, 10, (imputator.gop, imputator.gcp),
                              keep)
        else:
            prep = _read_prep(base_quality_threshold, cap_to_mapq, pcr_rate_factor, imputator.gcp, None, keep)
        out = np.empty(max(len(reads) * nh, 1), dtype=np.float64)
        rc = self._ctx.L.ghmm_compute_regions_raw(self._ctx.h, ctypes.byref(region), 1, ctypes.byref(prep),
                                                  out.ctypes.data_as(native._f64p))
        if rc == native.GHMM_ERR_ARG:
            raise ValueError(native.last_error(self._ctx.h))
        native.check(rc, self._ctx.h)
        self._last = out[:len(reads) * nh]
        return self._last

    def get_log_likelihood_array(self) -> np.ndarray | None:
        return self._last

    def close(self) -> None:
        self._ctx.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class MultiEngine:
    """One caller driving several GPUs (ghmm_multi_*): a context per listed device; each call's reads are cut into
    contiguous ranges of about equal cells, one per device, whose results land straight in their slice of the
    read-major output.  Devices may repeat (independent contexts on one GPU)."""

    def __init__(self, devices, max_threads: int = 0, use_double_precision: bool = False):
        self.L = native.lib()
        self.devices = [int(d) for d in devices]
        devs = (ctypes.c_int32 * len(self.devices))(*self.devices)
        a = native.Args(0, int(max_threads), int(use_double_precision), 0)
        h = ctypes.c_void_p()
        rc = self.L.ghmm_multi_create(devs, len(self.devices), ctypes.byref(a), ctypes.byref(h))
        if rc == native.GHMM_ERR_UNSUPPORTED:
            raise HardwareFeatureException(native.last_error(None))
        native.check(rc, None)
        self.h = h

    def _check(self, rc: int):
        if rc != native.GHMM_OK:
            buf = ctypes.create_string_buffer(1024)
            self.L.ghmm_multi_last_error(self.h, buf, len(buf))
            raise native.GhmmError(rc, buf.value.decode(errors="replace"))

    def compute(self, wl: Workload, out: np.ndarray | None = None) -> np.ndarray:
        """All pairs of wl (host buffers in, host results out), split over the devices."""
        if out is None:
            out = np.empty(wl.n_pairs, dtype=np.float64)
        regs = wl.as_regions()
        self._check(self.L.ghmm_multi_compute_regions(self.h, ctypes.cast(regs, ctypes.c_void_p), wl.n_regions,
                                                      out.ctypes.data_as(native._f64p)))
        return out

    def close(self):
        if self.h:
            self.L.ghmm_multi_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Engine:
    """Batched, device-resident use of the kernels (the batcher): one context, many regions."""

    def __init__(self, device: int = 0, max_threads: int = 0, use_double_precision: bool = False):
        self._ctx = _Context(PairHMMNativeArguments(max_threads, use_double_precision, device))
        self.L = self._ctx.L
        self.device = device
        self.double_precision = use_double_precision

    @property
    def handle(self):
        return self._ctx.h

    def stream_handle(self) -> int:
        return int(self.L.ghmm_stream(self._ctx.h) or 0)

    def compute(self, wl: Workload, via_regions: bool = False) -> np.ndarray:
        """Upload + forward + download (host buffers in, host results out)."""
        out = np.empty(wl.n_pairs, dtype=np.float64)
        if via_regions:
            regs = wl.as_regions()
            rc = self.L.ghmm_compute_regions(self._ctx.h, regs, wl.n_regions, out.ctypes.data_as(native._f64p))
        else:
            f = wl.as_flat()
            rc = self.L.ghmm_compute_flat(self._ctx.h, ctypes.byref(f), out.ctypes.data_as(native._f64p))
        native.check(rc, self._ctx.h)
        return out

    def set_tuning(self, max_rows_per_lane: int = 0, max_rows_per_lane_multi: int = 0, chunk_cols: int = 0,
                   route_fp64_below: int | None = None):
        """FP32 launch shape for batches created afterwards (0 keeps a field's default).  route_fp64_below (log10,
        < 0) sends reads expected to underflow the FP32 pass straight to FP64; None keeps the current setting."""
        if route_fp64_below is None:
            cur = native.Tuning()
            native.check(self.L.ghmm_get_tuning(self._ctx.h, ctypes.byref(cur)), self._ctx.h)
            route_fp64_below = cur.route_fp64_below
        t = native.Tuning(max_rows_per_lane, max_rows_per_lane_multi, chunk_cols, route_fp64_below)
        native.check(self.L.ghmm_set_tuning(self._ctx.h, ctypes.byref(t)), self._ctx.h)

    def get_tuning(self) -> tuple[int, int, int]:
        t = native.Tuning()
        native.check(self.L.ghmm_get_tuning(self._ctx.h, ctypes.byref(t)), self._ctx.h)
        return t.max_rows_per_lane, t.max_rows_per_lane_multi, t.chunk_cols

    def autotune(self, wl: Workload, **kw) -> dict:
        """Pick and set the fastest launch shape for workloads shaped like `wl` (gatk_gb300.autotune)."""
        from . import autotune

        return autotune.autotune(self, wl, device=self.device, **kw)

    def batch(self, wl: Workload, via_regions: bool = False) -> "Batch":
        return Batch(self, wl, via_regions)

    def compute_raw(self, wl: Workload, mapq, with_indel_quals: bool = True, base_quality_threshold: int = 18,
                    cap_to_mapq: bool = True, pcr_rate_factor: float = 3.0, gcp: int = 10,
                    dragstr=None) -> np.ndarray:
        """Likelihoods from raw reads, prepared on the device (PairHMMLikelihoodCalculationEngine.modifyReadQualities
        and the standard imputation, or with dragstr = (gop, gcp) tables of shape [max_period][max_repeats] the
        DRAGstr imputation); wl.quals are the raw base qualities, wl.ins / wl.dels the BI / BD tags."""
        from .workload import as_raw_regions

        out = np.empty(max(wl.n_pairs, 1), dtype=np.float64)
        regs = as_raw_regions(wl, mapq, with_indel_quals)
        p = _read_prep(base_quality_threshold, cap_to_mapq, pcr_rate_factor, gcp, dragstr, wl)
        native.check(self.L.ghmm_compute_regions_raw(self._ctx.h, regs, wl.n_regions, ctypes.byref(p),
                                                     out.ctypes.data_as(native._f64p)), self._ctx.h)
        return out[:wl.n_pairs]

    def pd_compute(self, wl: Workload, hap_pd: np.ndarray) -> np.ndarray:
        """PD-HMM log10 likelihoods of every pair (haplotypes with PD flags), host buffers in and out."""
        from .workload import as_pd_regions

        out = np.empty(max(wl.n_pairs, 1), dtype=np.float64)
        regs = as_pd_regions(wl, hap_pd)
        native.check(self.L.ghmm_pd_compute_regions(self._ctx.h, regs, wl.n_regions, out.ctypes.data_as(native._f64p)),
                     self._ctx.h)
        return out[:wl.n_pairs]

    def raw_batch(self, wl: Workload, mapq, with_indel_quals: bool = True, base_quality_threshold: int = 18,
                  cap_to_mapq: bool = True, pcr_rate_factor: float = 3.0, gcp: int = 10, dragstr=None) -> "Batch":
        p = _read_prep(base_quality_threshold, cap_to_mapq, pcr_rate_factor, gcp, dragstr, wl)
        return Batch(self, wl, raw=(mapq, with_indel_quals, p))

    def pd_batch(self, wl: Workload, hap_pd: np.ndarray) -> "Batch":
        return Batch(self, wl, pd=hap_pd)

    def pd_compute_raw(self, wl: Workload, hap_pd: np.ndarray, mapq, with_indel_quals: bool = True,
                       base_quality_threshold: int = 18, cap_to_mapq: bool = True, pcr_rate_factor: float = 3.0,
                       gcp: int = 10, dragstr=None) -> np.ndarray:
        """PD-HMM likelihoods from raw reads prepared on the device (ghmm_pd_compute_regions_raw); with dragstr =
        (gop, gcp) tables the DRAGEN-GATK chain of DRAGstr imputation and PD-HMM."""
        from .workload import as_pd_raw_regions

        out = np.empty(max(wl.n_pairs, 1), dtype=np.float64)
        regs = as_pd_raw_regions(wl, hap_pd, mapq, with_indel_quals)
        p = _read_prep(base_quality_threshold, cap_to_mapq, pcr_rate_factor, gcp, dragstr, wl)
        native.check(self.L.ghmm_pd_compute_regions_raw(self._ctx.h, regs, wl.n_regions, ctypes.byref(p),
                                                        out.ctypes.data_as(native._f64p)), self._ctx.h)
        return out[:wl.n_pairs]

    def pd_raw_batch(self, wl: Workload, hap_pd: np.ndarray, mapq, with_indel_quals: bool = True,
                     base_quality_threshold: int = 18, cap_to_mapq: bool = True, pcr_rate_factor: float = 3.0,
                     gcp: int = 10, dragstr=None) -> "Batch":
        p = _read_prep(base_quality_threshold, cap_to_mapq, pcr_rate_factor, gcp, dragstr, wl)
        return Batch(self, wl, pd_raw=(hap_pd, mapq, with_indel_quals, p))

    def queue(self, batch_cells: int = 0) -> "Queue":
        return Queue(self, batch_cells)

    def raw_queue(self, wl_keep: Workload, batch_cells: int = 0, base_quality_threshold: int = 18,
                  cap_to_mapq: bool = True, pcr_rate_factor: float = 3.0, gcp: int = 10, dragstr=None) -> "Queue":
        """A queue of raw reads prepared on the device (ghmm_queue_create_raw); the preparation arguments are kept
        alive on wl_keep until the queue is created (the library copies them, tables included)."""
        p = _read_prep(base_quality_threshold, cap_to_mapq, pcr_rate_factor, gcp, dragstr, wl_keep)
        return Queue(self, batch_cells, raw_prep=p)

    def measure_peaks(self):
        a, b, c = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        native.check(self.L.ghmm_measure_peaks(self._ctx.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)),
                     self._ctx.h)
        return {"fp32_tflops": a.value, "fp32x2_tflops": b.value, "fp64_tflops": c.value}

    def debug_tables(self):
        err = np.zeros(256)
        prob = np.zeros(256)
        m2m = np.zeros(128 * 128)
        native.check(self.L.ghmm_debug_tables(self._ctx.h, err.ctypes.data_as(native._f64p),
                                              prob.ctypes.data_as(native._f64p), m2m.ctypes.data_as(native._f64p)),
                     self._ctx.h)
        return err, prob, m2m.reshape(128, 128)

    def close(self):
        self._ctx.close()


class Batch:
    """A device-resident batch: inputs uploaded once; forward() reruns the kernels on them."""

    def __init__(self, engine: Engine, wl: Workload, via_regions: bool = False, pd=None, raw=None, pd_raw=None):
        self.engine = engine
        self.wl = wl
        h = ctypes.c_void_p()
        if pd_raw is not None:
            from .workload import as_pd_raw_regions

            hap_pd, mapq, with_indel, prep = pd_raw
            regs = as_pd_raw_regions(wl, hap_pd, mapq, with_indel)
            rc = engine.L.ghmm_pd_batch_create_raw(engine.handle, regs, wl.n_regions, ctypes.byref(prep),
                                                   ctypes.byref(h))
        elif raw is not None:
            from .workload import as_raw_regions

            mapq, with_indel, prep = raw
            regs = as_raw_regions(wl, mapq, with_indel)
            rc = engine.L.ghmm_batch_create_raw(engine.handle, regs, wl.n_regions, ctypes.byref(prep), ctypes.byref(h))
        elif pd is not None:
            from .workload import as_pd_regions

            regs = as_pd_regions(wl, pd)
            rc = engine.L.ghmm_pd_batch_create(engine.handle, regs, wl.n_regions, ctypes.byref(h))
        elif via_regions:
            regs = wl.as_regions()
            rc = engine.L.ghmm_batch_create(engine.handle, regs, wl.n_regions, ctypes.byref(h))
        else:
            f = wl.as_flat()
            rc = engine.L.ghmm_batch_create_flat(engine.handle, ctypes.byref(f), ctypes.byref(h))
        native.check(rc, engine.handle)
        self.h = h

    def forward(self, mode: int = native.MODE_FP32_RERUN) -> None:
        native.check(self.engine.L.ghmm_batch_forward(self.engine.handle, self.h, mode), self.engine.handle)

    def results(self) -> np.ndarray:
        out = np.empty(self.wl.n_pairs, dtype=np.float64)
        native.check(self.engine.L.ghmm_batch_results(self.engine.handle, self.h, out.ctypes.data_as(native._f64p)),
                     self.engine.handle)
        return out

    def postprocess(self, cap: float = -4.5, symmetric: bool = True, reference_hap=None, expected_error_rate: float = 0.02,
                    dynamic: bool = False, scale: float = 1.0) -> np.ndarray:
        """Normalise the last forward's likelihoods and flag poorly modelled reads on the device
        (PairHMMLikelihoodCalculationEngine.computeReadLikelihoods' last two steps); returns keep flags per read.
        cap is log10globalReadMismappingRate (GATK default -4.5: Phred 45)."""
        ref = None
        if reference_hap is not None:
            ref = np.ascontiguousarray(reference_hap, dtype=np.int32)
        p = native.Postprocess(float(cap), int(symmetric), int(dynamic), float(expected_error_rate), float(scale),
                               ref.ctypes.data if ref is not None else None)
        keep = np.empty(max(self.wl.n_reads, 1), dtype=np.uint8)
        native.check(self.engine.L.ghmm_batch_postprocess(self.engine.handle, self.h, ctypes.byref(p), keep.ctypes.data),
                     self.engine.handle)
        return keep[:self.wl.n_reads]

    def read_planes(self):
        """The five read planes as the kernels see them: (bases, quals, ins, dels, gcp)."""
        n = len(self.wl.bases)
        planes = [np.empty(max(n, 1), dtype=np.uint8) for _ in range(5)]
        native.check(self.engine.L.ghmm_batch_read_planes(self.engine.handle, self.h, *[p.ctypes.data for p in planes]),
                     self.engine.handle)
        return tuple(p[:n] for p in planes)

    def stats(self) -> dict:
        s = native.Stats()
        native.check(self.engine.L.ghmm_batch_stats(self.engine.handle, self.h, ctypes.byref(s)), self.engine.handle)
        return {k: getattr(s, k) for k, _ in native.Stats._fields_ if k != "reserved"}

    def close(self):
        if self.h:
            self.engine.L.ghmm_batch_destroy(self.engine.handle, self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Queue:
    """Streaming queue: push regions one at a time as they arrive; results land in the caller's arrays.

    ``push`` copies the region's inputs before it returns; the output array must stay alive (and is held
    here) until ``flush`` returns.
    """

    def __init__(self, engine: Engine, batch_cells: int = 0, raw_prep: native.ReadPrep | None = None):
        self.engine = engine
        h = ctypes.c_void_p()
        if raw_prep is None:
            rc = engine.L.ghmm_queue_create(engine.handle, int(batch_cells), ctypes.byref(h))
        else:
            rc = engine.L.ghmm_queue_create_raw(engine.handle, int(batch_cells), ctypes.byref(raw_prep), ctypes.byref(h))
        native.check(rc, engine.handle)
        self.h = h
        self.raw = raw_prep is not None
        self._keep: list = []

    def push_raw(self, wl: Workload, mapq, with_indel_quals: bool = True, out: np.ndarray | None = None) -> np.ndarray:
        """Push every region of a workload as raw reads (one push per region) into a raw queue; wl.quals are the raw
        base qualities, wl.ins / wl.dels the BI / BD tags (or none with with_indel_quals False)."""
        from .workload import as_raw_regions

        regs = as_raw_regions(wl, mapq, with_indel_quals)
        if out is None:
            out = np.empty(wl.n_pairs, dtype=np.float64)
        size = ctypes.sizeof(native.RawRegion)
        oo = wl.out_off
        for g in range(wl.n_regions):
            rc = self.engine.L.ghmm_queue_push_raw(self.h, regs + g * size, 1,
                                                   out.ctypes.data + int(oo[g]) * 8 if oo[g + 1] > oo[g] else None)
            native.check(rc, self.engine.handle)
        self._keep.append((out, wl))
        return out

    def push_regions(self, regions, n_regions: int, out: np.ndarray, keep=None) -> None:
        """Push n_regions ghmm_region structs starting at ``regions`` (a ctypes pointer); out is float64."""
        assert out.dtype == np.float64 and out.flags.c_contiguous
        rc = self.engine.L.ghmm_queue_push(self.h, ctypes.cast(regions, ctypes.c_void_p), int(n_regions),
                                           out.ctypes.data if out.size else None)
        self._keep.append(out)
        native.check(rc, self.engine.handle)

    def push(self, wl: Workload, out: np.ndarray | None = None) -> np.ndarray:
        """Push every region of a workload (one push per region); returns the output array."""
        regs = wl.as_regions()
        if out is None:
            out = np.empty(wl.n_pairs, dtype=np.float64)
        size = ctypes.sizeof(native.Region)
        base = ctypes.cast(regs, ctypes.c_void_p).value
        oo = wl.out_off
        for g in range(wl.n_regions):
            rc = self.engine.L.ghmm_queue_push(self.h, base + g * size, 1,
                                               out.ctypes.data + int(oo[g]) * 8 if oo[g + 1] > oo[g] else None)
            native.check(rc, self.engine.handle)
        self._keep.append((out, regs))
        return out

    def flush(self) -> None:
        rc = self.engine.L.ghmm_queue_flush(self.h)
        self._keep.clear()
        native.check(rc, self.engine.handle)

    def info(self) -> dict:
        i = native.QueueInfo()
        native.check(self.engine.L.ghmm_queue_get_info(self.h, ctypes.byref(i)), self.engine.handle)
        return {k: getattr(i, k) for k, _ in native.QueueInfo._fields_}

    def close(self) -> None:
        if self.h:
            rc = self.engine.L.ghmm_queue_destroy(self.h)
            self.h = None
            self._keep.clear()
            native.check(rc, self.engine.handle)

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
