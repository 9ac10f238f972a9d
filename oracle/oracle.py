"""ctypes binding of the CPU oracle (oracle/pairhmm_oracle.c, oracle_grad.c, pdhmm_oracle.c, sw_oracle.c,
readprep_oracle.c).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()`` as the
checker, and by the cpu_baseline / ``--impl reference`` leg of bench.py.  The product
package (gatk_gb300) never imports this module.

The C sources restate GATK's LoglessPairHMM / Log10PairHMM / PairHMMModel /
QualityUtils / MathUtils.JacobianLogTable, LoglessPDPairHMM, SmithWatermanJavaAligner and the read preparation
(modifyReadQualities, the PCR indel model, the DRAGstr imputation);
the file:line citations are in their headers.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None

_u8p = ctypes.POINTER(ctypes.c_uint8)
_i64p = ctypes.POINTER(ctypes.c_int64)
_f64p = ctypes.POINTER(ctypes.c_double)


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP, -ffp-contract=off)."""
    srcs = [os.path.join(_HERE, f) for f in ("pairhmm_oracle.c", "oracle_grad.c", "pdhmm_oracle.c", "sw_oracle.c",
                                            "readprep_oracle.c", "Makefile")]
    if not force and os.path.exists(_LIB_PATH):
        if os.path.getmtime(_LIB_PATH) >= max(os.path.getmtime(s) for s in srcs):
            return _LIB_PATH
    subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        L.oracle_logless.restype = ctypes.c_double
        L.oracle_logless.argtypes = [_u8p, ctypes.c_int, _u8p, _u8p, _u8p, _u8p, _u8p, ctypes.c_int, ctypes.c_int]
        L.oracle_log10_hmm.restype = ctypes.c_double
        L.oracle_log10_hmm.argtypes = [_u8p, ctypes.c_int, _u8p, _u8p, _u8p, _u8p, _u8p, ctypes.c_int,
                                       ctypes.c_int, ctypes.c_int]
        L.oracle_approx_log10_sum_log10.restype = ctypes.c_double
        L.oracle_approx_log10_sum_log10.argtypes = [ctypes.c_double, ctypes.c_double]
        L.oracle_match_to_match_prob.restype = ctypes.c_double
        L.oracle_match_to_match_prob.argtypes = [ctypes.c_int, ctypes.c_int]
        L.oracle_match_to_match_prob_log10.restype = ctypes.c_double
        L.oracle_match_to_match_prob_log10.argtypes = [ctypes.c_int, ctypes.c_int]
        L.oracle_qual_to_error_prob.restype = ctypes.c_double
        L.oracle_qual_to_error_prob.argtypes = [ctypes.c_int]
        L.oracle_qual_to_prob.restype = ctypes.c_double
        L.oracle_qual_to_prob.argtypes = [ctypes.c_int]
        L.oracle_qual_to_trans_probs.restype = None
        L.oracle_qual_to_trans_probs.argtypes = [_f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_qual_to_trans_probs_log10.restype = None
        L.oracle_qual_to_trans_probs_log10.argtypes = [_f64p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.oracle_validate_read.restype = ctypes.c_int
        L.oracle_validate_read.argtypes = [_u8p, _u8p, _u8p, _u8p, ctypes.c_int]
        L.oracle_compute_regions.restype = ctypes.c_int64
        L.oracle_compute_regions.argtypes = [ctypes.c_int32, _i64p, _i64p, _i64p, _u8p, _u8p, _u8p, _u8p, _u8p,
                                             _i64p, _u8p, _i64p, _f64p, ctypes.c_int]
        L.oracle_compute_pairs.restype = None
        L.oracle_compute_pairs.argtypes = [ctypes.c_int64, _i64p, _i64p, _i64p, _u8p, _u8p, _u8p, _u8p, _u8p,
                                           _i64p, _u8p, _f64p, ctypes.c_int]
        L.oracle_jacobian_size.restype = ctypes.c_int
        L.oracle_jacobian_value.restype = ctypes.c_double
        L.oracle_jacobian_value.argtypes = [ctypes.c_int]
        L.oracle_initial_condition_log10.restype = ctypes.c_double
        L.oracle_num_threads.restype = ctypes.c_int
        L.oracle_cont_forward.restype = ctypes.c_double
        L.oracle_cont_forward.argtypes = [_u8p, ctypes.c_int, _u8p, _u8p, _f64p, _f64p, ctypes.c_int]
        L.oracle_cont_grad.restype = ctypes.c_double
        L.oracle_cont_grad.argtypes = [_u8p, ctypes.c_int, _u8p, _u8p, _f64p, _f64p, ctypes.c_int, _f64p, _f64p]
        L.oracle_pd_logless.restype = ctypes.c_double
        L.oracle_pd_logless.argtypes = [_u8p, _u8p, ctypes.c_int, _u8p, _u8p, _u8p, _u8p, _u8p, ctypes.c_int,
                                        ctypes.POINTER(ctypes.c_int)]
        L.oracle_pd_compute_pairs.restype = ctypes.c_int64
        L.oracle_pd_compute_pairs.argtypes = [ctypes.c_int64, _i64p, _i64p, _i64p, _u8p, _u8p, _u8p, _u8p, _u8p,
                                              _i64p, _u8p, _u8p, _f64p, ctypes.c_int]
        _i32p = ctypes.POINTER(ctypes.c_int32)
        _u32p = ctypes.POINTER(ctypes.c_uint32)
        L.sw_oracle_align.restype = ctypes.c_int
        L.sw_oracle_align.argtypes = [_u8p, ctypes.c_int, _u8p, ctypes.c_int, _i32p, ctypes.c_int, ctypes.c_int, _u32p,
                                      ctypes.c_int, _i32p, _i32p]
        L.sw_oracle_align_batch.restype = ctypes.c_int
        L.sw_oracle_align_batch.argtypes = [ctypes.c_int64, _u8p, _i64p, _i32p, _u8p, _i64p, _i32p, _i32p, ctypes.c_int,
                                            ctypes.c_int, _u32p, _i64p, _i32p, _i32p, ctypes.c_int]
        L.rp_prepare_reads.restype = ctypes.c_int
        L.rp_prepare_reads.argtypes = [ctypes.c_int64, _i64p, _u8p, _u8p, _u8p, _u8p, _i32p, ctypes.c_int, ctypes.c_int,
                                       ctypes.c_double, ctypes.c_int, _f64p, _f64p, ctypes.c_int, ctypes.c_int, _u8p,
                                       _u8p, _u8p, _u8p, ctypes.c_int]
        _lib = L
    return _lib


def _u8(a) -> np.ndarray:
    if isinstance(a, (bytes, bytearray)):
        return np.frombuffer(bytes(a), dtype=np.uint8).copy()
    return np.ascontiguousarray(np.asarray(a, dtype=np.uint8))


def _p(a: np.ndarray, t):
    return a.ctypes.data_as(t)


def logless(hap, read, quals, ins, dels, gcp, tristate: bool = True) -> float:
    """LoglessPairHMM log10 likelihood of one pair (FP64)."""
    h, r, q, i, d, g = (_u8(x) for x in (hap, read, quals, ins, dels, gcp))
    return lib().oracle_logless(_p(h, _u8p), len(h), _p(r, _u8p), _p(q, _u8p), _p(i, _u8p), _p(d, _u8p),
                                _p(g, _u8p), len(r), int(tristate))


def log10_hmm(hap, read, quals, ins, dels, gcp, tristate: bool = True, exact: bool = True) -> float:
    """Log10PairHMM (EXACT when exact=True, ORIGINAL otherwise)."""
    h, r, q, i, d, g = (_u8(x) for x in (hap, read, quals, ins, dels, gcp))
    return lib().oracle_log10_hmm(_p(h, _u8p), len(h), _p(r, _u8p), _p(q, _u8p), _p(i, _u8p), _p(d, _u8p),
                                  _p(g, _u8p), len(r), int(tristate), int(exact))


def trans_probs(ins: int, dels: int, gcp: int, log10: bool = False) -> np.ndarray:
    out = np.zeros(6, dtype=np.float64)
    f = lib().oracle_qual_to_trans_probs_log10 if log10 else lib().oracle_qual_to_trans_probs
    f(_p(out, _f64p), ins, dels, gcp)
    return out


def compute_workload(wl, threads: int = 0) -> np.ndarray:
    """All pairs of a flat workload (gatk_gb300.workload.Workload layout), read-major per region."""
    L = lib()
    out = np.empty(int(wl.out_off[-1]), dtype=np.float64)
    L.oracle_compute_regions(wl.n_regions, _p(wl.region_read_off, _i64p), _p(wl.region_hap_off, _i64p),
                             _p(wl.read_off, _i64p), _p(wl.bases, _u8p), _p(wl.quals, _u8p), _p(wl.ins, _u8p),
                             _p(wl.dels, _u8p), _p(wl.gcp, _u8p), _p(wl.hap_off, _i64p), _p(wl.hap_bases, _u8p),
                             _p(wl.out_off, _i64p), _p(out, _f64p), int(threads))
    return out


def compute_pairs(wl, pair_read: np.ndarray, pair_hap: np.ndarray, threads: int = 0) -> np.ndarray:
    """Selected (read, haplotype) pairs of a flat workload; indices are global read/hap indices."""
    pr = np.ascontiguousarray(pair_read, dtype=np.int64)
    ph = np.ascontiguousarray(pair_hap, dtype=np.int64)
    out = np.empty(len(pr), dtype=np.float64)
    lib().oracle_compute_pairs(len(pr), _p(pr, _i64p), _p(ph, _i64p), _p(wl.read_off, _i64p), _p(wl.bases, _u8p),
                               _p(wl.quals, _u8p), _p(wl.ins, _u8p), _p(wl.dels, _u8p), _p(wl.gcp, _u8p),
                               _p(wl.hap_off, _i64p), _p(wl.hap_bases, _u8p), _p(out, _f64p), int(threads))
    return out


def cont_forward(hap, read, quals, g, c) -> float:
    h, r, q = (_u8(x) for x in (hap, read, quals))
    g = np.ascontiguousarray(g, dtype=np.float64)
    c = np.ascontiguousarray(c, dtype=np.float64)
    return lib().oracle_cont_forward(_p(h, _u8p), len(h), _p(r, _u8p), _p(q, _u8p), _p(g, _f64p), _p(c, _f64p),
                                     len(r))


def cont_grad(hap, read, quals, g, c):
    h, r, q = (_u8(x) for x in (hap, read, quals))
    g = np.ascontiguousarray(g, dtype=np.float64)
    c = np.ascontiguousarray(c, dtype=np.float64)
    dg = np.zeros(len(r), dtype=np.float64)
    dc = np.zeros(len(r), dtype=np.float64)
    v = lib().oracle_cont_grad(_p(h, _u8p), len(h), _p(r, _u8p), _p(q, _u8p), _p(g, _f64p), _p(c, _f64p), len(r),
                               _p(dg, _f64p), _p(dc, _f64p))
    return v, dg, dc


def num_threads() -> int:
    return lib().oracle_num_threads()


def pd_logless(hap, pd, read, quals, ins, dels, gcp) -> float:
    """LoglessPDPairHMM for one pair (pdhmm_oracle.c); raises ValueError where the reference throws."""
    h, f, r, q, i, d, g = (_u8(x) for x in (hap, pd, read, quals, ins, dels, gcp))
    err = ctypes.c_int(0)
    v = lib().oracle_pd_logless(_p(h, _u8p), _p(f, _u8p), len(h), _p(r, _u8p), _p(q, _u8p), _p(i, _u8p),
                                _p(d, _u8p), _p(g, _u8p), len(r), ctypes.byref(err))
    if err.value:
        raise ValueError("Found unexpected base in alt alleles")
    return v


def pd_compute_workload(wl, hap_pd: np.ndarray, threads: int = 0) -> np.ndarray:
    """Every pair of a workload whose haplotypes carry PD flags (hap_pd, parallel to hap_bases), read-major."""
    pr, ph = wl.pair_index()
    out = np.empty(len(pr), dtype=np.float64)
    if len(pr) == 0:
        return out
    pd = np.ascontiguousarray(hap_pd, dtype=np.uint8)
    pr = np.ascontiguousarray(pr, dtype=np.int64)
    ph = np.ascontiguousarray(ph, dtype=np.int64)
    bad = lib().oracle_pd_compute_pairs(len(pr), _p(pr, _i64p), _p(ph, _i64p), _p(wl.read_off, _i64p),
                                        _p(wl.bases, _u8p), _p(wl.quals, _u8p), _p(wl.ins, _u8p), _p(wl.dels, _u8p),
                                        _p(wl.gcp, _u8p), _p(wl.hap_off, _i64p), _p(wl.hap_bases, _u8p),
                                        _p(pd, _u8p), _p(out, _f64p), threads)
    if bad:
        raise ValueError(f"{bad} pairs hit 'Found unexpected base in alt alleles'")
    return out


_i32p = ctypes.POINTER(ctypes.c_int32)
_u32p = ctypes.POINTER(ctypes.c_uint32)


def sw_align(ref, alt, params, strategy: int, shortcut: bool = True):
    """Smith-Waterman of alt against ref (sw_oracle.c): (BAM-encoded cigar ops as a list, alignment offset)."""
    r, a = _u8(ref), _u8(alt)
    prm = np.ascontiguousarray(params, dtype=np.int32)
    ops = np.zeros(2 * len(a) + 4, dtype=np.uint32)
    n_ops, off = ctypes.c_int32(0), ctypes.c_int32(0)
    st = lib().sw_oracle_align(_p(r, _u8p), len(r), _p(a, _u8p), len(a), _p(prm, _i32p), strategy, int(shortcut),
                               _p(ops, _u32p), len(ops), ctypes.byref(n_ops), ctypes.byref(off))
    if st != 0:
        raise ValueError(f"sw_oracle_align status {st}")
    return [int(x) for x in ops[:n_ops.value]], off.value


def sw_align_pairs(ref_plane, ref_off, ref_len, alt_plane, alt_off, alt_len, params, strategy: int,
                   shortcut: bool = True, threads: int = 0):
    """Many alignments over all host threads: (ops, ops_start, n_ops, offset); pair p's BAM-encoded ops are
    ops[ops_start[p]:ops_start[p] + n_ops[p]]."""
    n = len(ref_off)
    ref_plane, alt_plane = _u8(ref_plane), _u8(alt_plane)
    ref_off = np.ascontiguousarray(ref_off, dtype=np.int64)
    alt_off = np.ascontiguousarray(alt_off, dtype=np.int64)
    ref_len = np.ascontiguousarray(ref_len, dtype=np.int32)
    alt_len = np.ascontiguousarray(alt_len, dtype=np.int32)
    prm = np.ascontiguousarray(params, dtype=np.int32)
    cap = 2 * alt_len.astype(np.int64) + 4
    start = np.zeros(n, dtype=np.int64)
    if n > 1:
        start[1:] = np.cumsum(cap)[:-1]
    ops = np.zeros(int(cap.sum()) if n else 1, dtype=np.uint32)
    n_ops = np.zeros(n, dtype=np.int32)
    off = np.zeros(n, dtype=np.int32)
    if n == 0:
        return ops, start, n_ops, off
    st = lib().sw_oracle_align_batch(n, _p(ref_plane, _u8p), _p(ref_off, _i64p), _p(ref_len, _i32p),
                                     _p(alt_plane, _u8p), _p(alt_off, _i64p), _p(alt_len, _i32p), _p(prm, _i32p),
                                     strategy, int(shortcut), _p(ops, _u32p), _p(start, _i64p), _p(n_ops, _i32p),
                                     _p(off, _i32p), threads)
    if st != 0:
        raise ValueError(f"sw_oracle_align_batch status {st}")
    return ops, start, n_ops, off


def prepare_reads(read_off, bases, quals, ins, dels, mapq, threshold: int = 18, cap_to_mapq: bool = True,
                  rate_factor: float = 0.0, gcp: int = 10, dragstr=None, threads: int = 0):
    """readprep_oracle.c over reads laid back to back at read_off: the (quals, ins, dels, gcp) planes, as
    oracle/readprep.py's prepare_read gives them read by read.  ins / dels None: 45 everywhere; dragstr = (gop, gcp)
    tables [max_period][max_repeats] or None."""
    read_off = np.ascontiguousarray(read_off, dtype=np.int64)
    n_reads = len(read_off) - 1
    bases, quals = _u8(bases), _u8(quals)
    ins_a = None if ins is None else _u8(ins)
    dels_a = None if dels is None else _u8(dels)
    mq = np.ascontiguousarray(mapq, dtype=np.int32)
    outs = [np.zeros(max(len(bases), 1), dtype=np.uint8) for _ in range(4)]
    gop_t = gcp_t = None
    maxp = maxr = 0
    if dragstr is not None:
        gop_t = np.ascontiguousarray(dragstr[0], dtype=np.float64)
        gcp_t = np.ascontiguousarray(dragstr[1], dtype=np.float64)
        maxp, maxr = gop_t.shape
    st = lib().rp_prepare_reads(n_reads, _p(read_off, _i64p), _p(bases, _u8p), _p(quals, _u8p),
                                _p(ins_a, _u8p) if ins_a is not None else None,
                                _p(dels_a, _u8p) if dels_a is not None else None, _p(mq, _i32p), int(threshold),
                                int(cap_to_mapq), float(rate_factor), int(gcp),
                                _p(gop_t, _f64p) if gop_t is not None else None,
                                _p(gcp_t, _f64p) if gcp_t is not None else None, int(maxp), int(maxr),
                                *[_p(o, _u8p) for o in outs], int(threads))
    if st != 0:
        raise ValueError(f"rp_prepare_reads status {st}")
    return tuple(o[:len(bases)] for o in outs)
