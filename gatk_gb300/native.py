"""ctypes binding of libghmm.so (include/ghmm.h, ghmm_sw.h, ghmm_calib.h) and of the synthetic workload
generator libghmm_synth.so (include/ghmm_synth.h).

The library is the product: there is no Python or CPU fallback.  ``lib()`` builds it in-tree if it
is missing and raises if that fails; compute calls raise ``GhmmError`` with the library's message
when the device is absent or a call fails.  The generator is test and benchmark input, kept in a library
of its own (``synth_lib()``) so that loading it does not load the product.
"""
from __future__ import annotations

import ctypes
import threading

from . import build as _build

GHMM_OK = 0
GHMM_ERR_ARG = 1
GHMM_ERR_STATE = 2
GHMM_ERR_CUDA = 3
GHMM_ERR_UNSUPPORTED = 4
GHMM_ERR_RESULT = 5
GHMM_ERR_NOMEM = 6
GHMM_ERR_TIMEOUT = 7

MODE_FP32_RERUN = 0
MODE_FP64 = 1
MODE_PD = 3
MODE_PD_FP32 = 4
INJECT_REFUSE_ALLOCATIONS = 1
INJECT_FP64_RERUN_EVERY = 2
FP64_RESCALED_FLOOR = -560.0  # GHMM_FP64_RESCALED_FLOOR
MODE_PLAIN_FP64 = 2

FP32_RERUN_THRESHOLD = 1e-28

_u8p = ctypes.POINTER(ctypes.c_uint8)
_i64p = ctypes.POINTER(ctypes.c_int64)
_i32p = ctypes.POINTER(ctypes.c_int32)
_f64p = ctypes.POINTER(ctypes.c_double)
_f32p = ctypes.POINTER(ctypes.c_float)


class GhmmError(RuntimeError):
    def __init__(self, code: int, message: str):
        super().__init__(f"[{code}] {message}")
        self.code = code


class Args(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int32), ("max_threads", ctypes.c_int32),
                ("use_double_precision", ctypes.c_int32), ("flags", ctypes.c_int32)]


class Tuning(ctypes.Structure):
    _fields_ = [("max_rows_per_lane", ctypes.c_int32), ("max_rows_per_lane_multi", ctypes.c_int32),
                ("chunk_cols", ctypes.c_int32), ("route_fp64_below", ctypes.c_int32)]


class Read(ctypes.Structure):
    _fields_ = [("bases", _u8p), ("quals", _u8p), ("ins_gop", _u8p), ("del_gop", _u8p), ("gcp", _u8p),
                ("length", ctypes.c_int32)]


class Hap(ctypes.Structure):
    _fields_ = [("bases", _u8p), ("length", ctypes.c_int32)]


class Region(ctypes.Structure):
    _fields_ = [("reads", ctypes.POINTER(Read)), ("n_reads", ctypes.c_int32), ("haps", ctypes.POINTER(Hap)),
                ("n_haps", ctypes.c_int32)]


class Flat(ctypes.Structure):
    _fields_ = [("n_regions", ctypes.c_int64), ("region_read_off", _i64p), ("region_hap_off", _i64p),
                ("read_off", _i64p), ("bases", _u8p), ("quals", _u8p), ("ins_gop", _u8p), ("del_gop", _u8p),
                ("gcp", _u8p), ("hap_off", _i64p), ("hap_bases", _u8p), ("out_off", _i64p)]


class Stats(ctypes.Structure):
    _fields_ = [("n_pairs", ctypes.c_int64), ("n_cells", ctypes.c_int64), ("n_rerun", ctypes.c_int64),
                ("n_fp64_direct", ctypes.c_int64), ("n_tasks_fp32", ctypes.c_int64), ("n_launches", ctypes.c_int32),
                ("reserved", ctypes.c_int32), ("ms_fp32", ctypes.c_double), ("ms_fp64", ctypes.c_double),
                ("ms_plain", ctypes.c_double), ("ms_total", ctypes.c_double), ("h2d_bytes", ctypes.c_int64),
                ("d2h_bytes", ctypes.c_int64), ("ms_host_marshal", ctypes.c_double),
                ("ms_host_tasks", ctypes.c_double), ("n_fp64_exact", ctypes.c_int64), ("ms_prep", ctypes.c_double),
                ("n_cells_fp64_direct", ctypes.c_int64)]


class RawRead(ctypes.Structure):
    _fields_ = [("bases", ctypes.c_void_p), ("quals", ctypes.c_void_p), ("ins_quals", ctypes.c_void_p),
                ("del_quals", ctypes.c_void_p), ("length", ctypes.c_int32), ("mapping_quality", ctypes.c_int32)]


class PdRawRegion(ctypes.Structure):
    _fields_ = [("reads", ctypes.c_void_p), ("n_reads", ctypes.c_int32), ("haps", ctypes.c_void_p),
                ("n_haps", ctypes.c_int32)]


class RawRegion(ctypes.Structure):
    _fields_ = [("reads", ctypes.c_void_p), ("n_reads", ctypes.c_int32), ("haps", ctypes.c_void_p),
                ("n_haps", ctypes.c_int32)]


class Dragstr(ctypes.Structure):
    _fields_ = [("max_period", ctypes.c_int32), ("max_repeats", ctypes.c_int32), ("gop", ctypes.c_void_p),
                ("gcp", ctypes.c_void_p)]


class ReadPrep(ctypes.Structure):
    _fields_ = [("base_quality_threshold", ctypes.c_int32), ("cap_to_mapq", ctypes.c_int32),
                ("pcr_rate_factor", ctypes.c_double), ("gcp", ctypes.c_int32), ("reserved", ctypes.c_int32),
                ("dragstr", ctypes.c_void_p)]


class PdHap(ctypes.Structure):
    _fields_ = [("bases", ctypes.c_void_p), ("pd_bases", ctypes.c_void_p), ("length", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


class PdRegion(ctypes.Structure):
    _fields_ = [("reads", ctypes.c_void_p), ("n_reads", ctypes.c_int32), ("haps", ctypes.c_void_p),
                ("n_haps", ctypes.c_int32)]


class Postprocess(ctypes.Structure):
    _fields_ = [("max_likelihood_difference_cap", ctypes.c_double), ("symmetric", ctypes.c_int32),
                ("dynamic_disqualification", ctypes.c_int32), ("expected_error_rate_per_base", ctypes.c_double),
                ("read_disqualification_scale", ctypes.c_double), ("reference_hap", ctypes.c_void_p)]


class QueueInfo(ctypes.Structure):
    _fields_ = [("n_regions", ctypes.c_int64), ("n_pairs", ctypes.c_int64), ("n_cells", ctypes.c_int64),
                ("n_cells_fp64_direct", ctypes.c_int64), ("n_rerun", ctypes.c_int64), ("n_fp64_direct", ctypes.c_int64),
                ("n_batches", ctypes.c_int64), ("n_launches", ctypes.c_int64), ("h2d_bytes", ctypes.c_int64),
                ("d2h_bytes", ctypes.c_int64), ("ms_fp32", ctypes.c_double), ("ms_fp64", ctypes.c_double),
                ("ms_host_marshal", ctypes.c_double), ("ms_host_tasks", ctypes.c_double),
                ("n_fp64_exact", ctypes.c_int64)]


class DevPairs(ctypes.Structure):
    _fields_ = [("bases", ctypes.c_void_p), ("quals", ctypes.c_void_p), ("ins_gop", ctypes.c_void_p),
                ("del_gop", ctypes.c_void_p), ("gcp", ctypes.c_void_p), ("read_off", ctypes.c_void_p),
                ("hap_bases", ctypes.c_void_p), ("hap_off", ctypes.c_void_p), ("pair_read", ctypes.c_void_p),
                ("pair_hap", ctypes.c_void_p), ("n_pairs", ctypes.c_int64), ("max_hap_len", ctypes.c_int32),
                ("reserved", ctypes.c_int32)]


NOALLOC_MAX_HAP_LEN = 2048


class MultiSlice(ctypes.Structure):
    _fields_ = [("read_begin", ctypes.c_int64), ("read_end", ctypes.c_int64), ("out_begin", ctypes.c_int64),
                ("out_end", ctypes.c_int64), ("cells", ctypes.c_int64)]


class CalibBatch(ctypes.Structure):
    _fields_ = [("bases", ctypes.c_void_p), ("quals", ctypes.c_void_p), ("read_off", ctypes.c_void_p),
                ("hap_bases", ctypes.c_void_p), ("hap_off", ctypes.c_void_p), ("pair_read", ctypes.c_void_p),
                ("pair_hap", ctypes.c_void_p), ("gap_open", ctypes.c_void_p), ("gap_cont", ctypes.c_void_p),
                ("n_pairs", ctypes.c_int64), ("max_read_len", ctypes.c_int32), ("max_hap_len", ctypes.c_int32)]


class SynthArrays(ctypes.Structure):
    _fields_ = [("n_regions", ctypes.c_int64), ("n_reads", ctypes.c_int64), ("n_haps", ctypes.c_int64),
                ("read_bytes", ctypes.c_int64), ("hap_bytes", ctypes.c_int64), ("n_out", ctypes.c_int64),
                ("region_read_off", _i64p), ("region_hap_off", _i64p), ("read_off", _i64p), ("hap_off", _i64p),
                ("out_off", _i64p), ("bases", _u8p), ("quals", _u8p), ("ins", _u8p), ("dels", _u8p), ("gcp", _u8p),
                ("hap_bases", _u8p)]


# Smith-Waterman (include/ghmm_sw.h)
SW_SOFTCLIP, SW_INDEL, SW_LEADING_INDEL, SW_IGNORE = 0, 1, 2, 3
SW_SUBSTRING_SHORTCUT = 1
CIGAR_M, CIGAR_I, CIGAR_D, CIGAR_S = 0, 1, 2, 4
SW_MAX_LEN = 1 << 20
SW_OPT_INT32_ONLY = 1


class SwParams(ctypes.Structure):
    _fields_ = [("match_value", ctypes.c_int32), ("mismatch_penalty", ctypes.c_int32),
                ("gap_open_penalty", ctypes.c_int32), ("gap_extend_penalty", ctypes.c_int32)]


class SwPair(ctypes.Structure):
    _fields_ = [("ref", ctypes.c_void_p), ("alt", ctypes.c_void_p), ("ref_len", ctypes.c_int32),
                ("alt_len", ctypes.c_int32)]


class SwResult(ctypes.Structure):
    _fields_ = [("alignment_offset", ctypes.c_void_p), ("cigar_start", ctypes.c_void_p),
                ("cigar_len", ctypes.c_void_p), ("cigar_ops", ctypes.c_void_p), ("cigar_cap", ctypes.c_int64),
                ("cigar_total", ctypes.c_int64)]


class SwStats(ctypes.Structure):
    _fields_ = [("n_alignments", ctypes.c_int64), ("n_shortcut", ctypes.c_int64), ("cells", ctypes.c_int64),
                ("chunks", ctypes.c_int32), ("launches", ctypes.c_int32), ("ms_device", ctypes.c_double),
                ("ms_forward", ctypes.c_double), ("ms_total", ctypes.c_double), ("h2d_bytes", ctypes.c_int64),
                ("d2h_bytes", ctypes.c_int64), ("ms_host", ctypes.c_double), ("n_int16", ctypes.c_int64)]


# Every exported symbol and its signature (restype, argtypes).  The tests check that the library
# exports exactly the functions the public headers declare.
_SIGS = {
    "ghmm_load": (ctypes.c_int, []),
    "ghmm_initialize": (ctypes.c_int, [ctypes.POINTER(Args), ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_compute_likelihoods": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Read), ctypes.c_int32,
                                                ctypes.POINTER(Hap), ctypes.c_int32, _f64p]),
    "ghmm_done": (ctypes.c_int, [ctypes.c_void_p]),
    "ghmm_set_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tuning)]),
    "ghmm_get_tuning": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Tuning)]),
    "ghmm_autotune": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Flat), ctypes.POINTER(Tuning), ctypes.c_int32,
                                     ctypes.c_int32, ctypes.POINTER(Tuning), _f64p]),
    "ghmm_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "ghmm_compute_regions": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Region), ctypes.c_int32, _f64p]),
    "ghmm_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Region), ctypes.c_int32,
                                         ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_batch_create_flat": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Flat), ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_batch_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32]),
    "ghmm_batch_results": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, _f64p]),
    "ghmm_batch_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Stats)]),
    "ghmm_batch_destroy": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p]),
    "ghmm_compute_regions_raw": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                                ctypes.POINTER(ReadPrep), _f64p]),
    "ghmm_batch_create_raw": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                             ctypes.POINTER(ReadPrep), ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_batch_read_planes": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ghmm_pd_compute_likelihoods": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Read), ctypes.c_int32,
                                                   ctypes.POINTER(PdHap), ctypes.c_int32, _f64p]),
    "ghmm_pd_compute_regions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, _f64p]),
    "ghmm_pd_batch_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                            ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_pd_compute_regions_raw": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                                   ctypes.POINTER(ReadPrep), _f64p]),
    "ghmm_pd_batch_create_raw": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32,
                                                ctypes.POINTER(ReadPrep), ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_batch_postprocess": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(Postprocess),
                                              ctypes.c_void_p]),
    "ghmm_compute_flat": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(Flat), _f64p]),
    "ghmm_stream": (ctypes.c_void_p, [ctypes.c_void_p]),
    "ghmm_queue_create": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_queue_push": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "ghmm_debug_inject": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int64]),
    "ghmm_queue_create_raw": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64, ctypes.c_void_p,
                                             ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_queue_push_raw": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p]),
    "ghmm_queue_flush": (ctypes.c_int, [ctypes.c_void_p]),
    "ghmm_queue_get_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(QueueInfo)]),
    "ghmm_queue_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ghmm_measure_peaks": (ctypes.c_int, [ctypes.c_void_p, _f64p, _f64p, _f64p]),
    "ghmm_debug_tables": (ctypes.c_int, [ctypes.c_void_p, _f64p, _f64p, _f64p]),
    "ghmm_debug_pd_ops": (ctypes.c_int, [_u8p, _u8p, ctypes.c_int32, _u8p, _u8p]),
    "ghmm_debug_pipeline_cuts": (ctypes.c_int, [_i64p, ctypes.c_int64, _i64p, ctypes.c_int64, _i64p]),
    "ghmm_str_analyze": (ctypes.c_int, [_u8p, ctypes.c_int32, ctypes.c_int32, _i32p, _i32p, _i32p]),
    "ghmm_calib_forward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CalibBatch), ctypes.c_int32, ctypes.c_void_p]),
    "ghmm_calib_backward": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(CalibBatch), ctypes.c_int32, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "ghmm_multi_create": (ctypes.c_int, [_i32p, ctypes.c_int32, ctypes.POINTER(Args), ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_multi_compute_regions": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, _f64p]),
    "ghmm_multi_plan": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.POINTER(MultiSlice)]),
    "ghmm_multi_context": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_multi_last_error": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_char_p, ctypes.c_size_t]),
    "ghmm_multi_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "ghmm_forward_pairs_noalloc": (ctypes.c_int, [ctypes.c_int32, ctypes.POINTER(DevPairs), ctypes.c_void_p,
                                                  ctypes.c_void_p]),
    "ghmm_sw_align": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int32, ctypes.c_void_p, ctypes.c_int32,
                                     ctypes.POINTER(SwParams), ctypes.c_int32, ctypes.c_char_p, ctypes.c_int32, _i32p]),
    "ghmm_sw_cigar_bound": (ctypes.c_int64, [ctypes.POINTER(SwPair), ctypes.c_int32]),
    "ghmm_sw_align_batch": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SwPair), ctypes.c_int32,
                                           ctypes.POINTER(SwParams), ctypes.c_int32, ctypes.c_int32,
                                           ctypes.POINTER(SwResult)]),
    "ghmm_batch_realign": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(SwParams),
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(SwResult)]),
    "ghmm_sw_last_stats": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SwStats)]),
    "ghmm_sw_set_traceback_budget": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int64]),
    "ghmm_sw_measure_peak": (ctypes.c_int, [ctypes.c_void_p, _f64p]),
    "ghmm_sw_set_options": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
}

# The synthetic generator's symbols (include/ghmm_synth.h), exported by libghmm_synth.so.
_SYNTH_SIGS = {
    "ghmm_synth_default_regions": (ctypes.c_int64, [ctypes.c_int32]),
    "ghmm_synth_generate": (ctypes.c_int, [ctypes.c_int32, ctypes.c_uint64, ctypes.c_int64, ctypes.c_int64,
                                           ctypes.c_int32, ctypes.POINTER(ctypes.c_void_p)]),
    "ghmm_synth_view": (ctypes.c_int, [ctypes.c_void_p, ctypes.POINTER(SynthArrays)]),
    "ghmm_synth_free": (None, [ctypes.c_void_p]),
}

_lib = None
_synth = None
_lock = threading.Lock()


def lib_path() -> str:
    return _build.LIB


def lib():
    """Load libghmm.so (building it in-tree first if needed)."""
    global _lib
    with _lock:
        if _lib is None:
            path = _build.build()
            L = ctypes.CDLL(path)
            for name, (res, args) in _SIGS.items():
                f = getattr(L, name, None)
                if f is None:
                    raise ImportError(f"{path} does not export {name}")
                f.restype = res
                f.argtypes = args
            _lib = L
    return _lib


def synth_lib():
    """Load libghmm_synth.so, the synthetic workload generator (building it in-tree first if needed)."""
    global _synth
    with _lock:
        if _synth is None:
            _build.build()
            L = ctypes.CDLL(_build.SYNTH_LIB)
            for name, (res, args) in _SYNTH_SIGS.items():
                f = getattr(L, name, None)
                if f is None:
                    raise ImportError(f"{_build.SYNTH_LIB} does not export {name}")
                f.restype = res
                f.argtypes = args
            _synth = L
    return _synth


def exported_symbols():
    return sorted(_SIGS)


def synth_symbols():
    return sorted(_SYNTH_SIGS)


def last_error(ctx) -> str:
    buf = ctypes.create_string_buffer(1024)
    lib().ghmm_last_error(ctx, buf, len(buf))
    return buf.value.decode(errors="replace")


def check(code: int, ctx=None):
    if code != GHMM_OK:
        raise GhmmError(code, last_error(ctx))


def device_available() -> bool:
    return bool(lib().ghmm_load())
