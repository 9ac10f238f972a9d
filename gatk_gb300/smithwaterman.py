"""Host-side mirror of GATK's Smith-Waterman aligner interface, backed by the GB300 aligner (include/ghmm_sw.h).

Reference interface (paths inside the GATK repository, src/main/java/org/broadinstitute/hellbender/):
  SmithWatermanAligner.align(ref, alt, SWParameters, SWOverhangStrategy), close(), Implementation
      utils/smithwaterman/SmithWatermanAligner.java:14-87
  SWNativeAlignerWrapper.align: exact-substring shortcut, then the native binding       SWNativeAlignerWrapper.java:31-59
  SmithWatermanAlignment {getCigar(), getAlignmentOffset()}                              SmithWatermanAlignment.java
  SmithWatermanAlignmentConstants (parameter sets)                                       SmithWatermanAlignmentConstants.java:30-68
  SWParameters / SWOverhangStrategy (gatk-native-bindings 1.1.0)

Every alignment runs on the GPU through libghmm.so; there is no CPU path.
"""
from __future__ import annotations

import ctypes
import enum
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import native
from .pairhmm import HardwareFeatureException, PairHMMNativeArguments, _Context


class SWOverhangStrategy(enum.IntEnum):
    SOFTCLIP = native.SW_SOFTCLIP
    INDEL = native.SW_INDEL
    LEADING_INDEL = native.SW_LEADING_INDEL
    IGNORE = native.SW_IGNORE


@dataclass(frozen=True)
class SWParameters:
    match_value: int
    mismatch_penalty: int
    gap_open_penalty: int
    gap_extend_penalty: int

    def as_native(self) -> native.SwParams:
        return native.SwParams(self.match_value, self.mismatch_penalty, self.gap_open_penalty, self.gap_extend_penalty)


# SmithWatermanAlignmentConstants.java:30,38,52,68
ORIGINAL_DEFAULT = SWParameters(3, -1, -4, -3)
STANDARD_NGS = SWParameters(25, -50, -110, -6)
NEW_SW_PARAMETERS = SWParameters(200, -150, -260, -11)
ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS = SWParameters(10, -15, -30, -5)

_OP_CHARS = "MIDNSHP=X"


def cigar_text(ops: np.ndarray) -> str:
    """htsjdk TextCigarCodec.encode of BAM-encoded ops (length << 4 | op); '*' for none."""
    if len(ops) == 0:
        return "*"
    return "".join(f"{int(o) >> 4}{_OP_CHARS[int(o) & 15]}" for o in ops)


@dataclass
class SmithWatermanAlignment:
    cigar: str
    alignment_offset: int

    def get_cigar(self) -> str:
        return self.cigar

    def get_alignment_offset(self) -> int:
        return self.alignment_offset


@dataclass
class AlignmentBatch:
    """Batched results: alignment i is cigar_ops[cigar_start[i]:cigar_start[i] + cigar_len[i]] at offset[i]."""
    offset: np.ndarray
    cigar_start: np.ndarray
    cigar_len: np.ndarray
    cigar_ops: np.ndarray

    def __len__(self) -> int:
        return len(self.offset)

    def ops(self, i: int) -> np.ndarray:
        s = int(self.cigar_start[i])
        return self.cigar_ops[s:s + int(self.cigar_len[i])]

    def cigar(self, i: int) -> str:
        return cigar_text(self.ops(i))

    def alignment(self, i: int) -> SmithWatermanAlignment:
        return SmithWatermanAlignment(self.cigar(i), int(self.offset[i]))


def _u8(x) -> np.ndarray:
    if isinstance(x, (bytes, bytearray)):
        return np.frombuffer(bytes(x), dtype=np.uint8)
    return np.ascontiguousarray(np.asarray(x, dtype=np.uint8))


def _result(n: int, cap: int):
    off = np.empty(max(n, 1), dtype=np.int32)
    start = np.empty(max(n, 1), dtype=np.int64)
    length = np.empty(max(n, 1), dtype=np.int32)
    ops = np.empty(max(cap, 1), dtype=np.uint32)
    r = native.SwResult(off.ctypes.data, start.ctypes.data, length.ctypes.data, ops.ctypes.data, int(cap), 0)
    return r, off, start, length, ops


class SmithWatermanCudaAligner:
    """SmithWatermanAligner on the GPU: ``align`` is SWNativeAlignerWrapper.align with the GB300 binding behind it
    (the substring shortcut here, as the wrapper does, then ghmm_sw_align); ``align_many`` aligns a whole list of
    pairs in one call."""

    def __init__(self, device: int = 0, max_threads: int = 0):
        self._ctx = _Context(PairHMMNativeArguments(max_threads, False, device))

    @property
    def handle(self):
        return self._ctx.h

    def align(self, ref, alt, parameters: SWParameters = ORIGINAL_DEFAULT,
              overhang_strategy: SWOverhangStrategy = SWOverhangStrategy.SOFTCLIP) -> SmithWatermanAlignment:
        r, a = bytes(_u8(ref)), bytes(_u8(alt))
        if parameters is None or overhang_strategy is None:
            raise ValueError("parameters and overhang strategy must not be null")
        if overhang_strategy in (SWOverhangStrategy.SOFTCLIP, SWOverhangStrategy.IGNORE) and r and a:
            idx = r.rfind(a)  # Utils.lastIndexOf
            if idx != -1:
                return SmithWatermanAlignment(f"{len(a)}M", idx)
        return self.align_native(r, a, parameters, overhang_strategy)

    def align_native(self, ref, alt, parameters: SWParameters, overhang_strategy: SWOverhangStrategy):
        """SWAlignerNativeBinding.align: no shortcut."""
        r, a = _u8(ref), _u8(alt)
        buf = ctypes.create_string_buffer(2 * (len(a) + 4) * 8 + 16)
        off = ctypes.c_int32(0)
        p = parameters.as_native()
        rc = self._ctx.L.ghmm_sw_align(self._ctx.h, r.ctypes.data if len(r) else None, len(r),
                                       a.ctypes.data if len(a) else None, len(a), ctypes.byref(p),
                                       int(overhang_strategy), buf, len(buf), ctypes.byref(off))
        if rc == native.GHMM_ERR_ARG:
            raise ValueError(native.last_error(self._ctx.h))
        native.check(rc, self._ctx.h)
        return SmithWatermanAlignment(buf.value.decode(), off.value)

    def align_many(self, refs: Sequence, alts: Sequence, parameters: SWParameters = ORIGINAL_DEFAULT,
                   overhang_strategy: SWOverhangStrategy = SWOverhangStrategy.SOFTCLIP,
                   substring_shortcut: bool = True) -> AlignmentBatch:
        if len(refs) != len(alts):
            raise ValueError("refs and alts differ in length")
        n = len(refs)
        rs = [_u8(x) for x in refs]
        as_ = [_u8(x) for x in alts]
        pairs = (native.SwPair * max(n, 1))()
        for i in range(n):
            pairs[i] = native.SwPair(rs[i].ctypes.data if len(rs[i]) else None,
                                     as_[i].ctypes.data if len(as_[i]) else None, len(rs[i]), len(as_[i]))
        cap = int(self._ctx.L.ghmm_sw_cigar_bound(pairs, n))
        res, off, start, length, ops = _result(n, cap)
        p = parameters.as_native()
        rc = self._ctx.L.ghmm_sw_align_batch(self._ctx.h, pairs, n, ctypes.byref(p), int(overhang_strategy),
                                             native.SW_SUBSTRING_SHORTCUT if substring_shortcut else 0,
                                             ctypes.byref(res))
        if rc == native.GHMM_ERR_ARG:
            raise ValueError(native.last_error(self._ctx.h))
        native.check(rc, self._ctx.h)
        return AlignmentBatch(off[:n], start[:n], length[:n], ops[:res.cigar_total])

    def last_stats(self) -> dict:
        return sw_stats(self._ctx.L, self._ctx.h)

    def measure_peak(self) -> float:
        """Measured int32 max throughput in Tops/s (ghmm_sw_measure_peak)."""
        v = ctypes.c_double()
        native.check(self._ctx.L.ghmm_sw_measure_peak(self._ctx.h, ctypes.byref(v)), self._ctx.h)
        return v.value

    def set_int32_only(self, on: bool = True) -> None:
        """Run every alignment in the int32 kernel (by default bounded ones run two per warp in 16 bits)."""
        native.check(self._ctx.L.ghmm_sw_set_options(self._ctx.h, native.SW_OPT_INT32_ONLY if on else 0), self._ctx.h)

    def set_traceback_budget(self, nbytes: int) -> None:
        native.check(self._ctx.L.ghmm_sw_set_traceback_budget(self._ctx.h, int(nbytes)), self._ctx.h)

    def close(self) -> None:
        self._ctx.close()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Implementation(enum.Enum):
    """The SmithWatermanAligner.Implementation constant this package adds."""

    CUDA = "CUDA"

    def create_aligner(self, device: int = 0) -> SmithWatermanCudaAligner:
        """Raises HardwareFeatureException without a usable GPU, as SmithWatermanIntelAligner's constructor does
        without AVX (SmithWatermanIntelAligner.java:29-35)."""
        return SmithWatermanCudaAligner(device)


def sw_stats(L, h) -> dict:
    s = native.SwStats()
    native.check(L.ghmm_sw_last_stats(h, ctypes.byref(s)), h)
    return {k: getattr(s, k) for k, _ in native.SwStats._fields_}


def realign_batch(batch, hap_priority=None, parameters: SWParameters = ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS):
    """ghmm_batch_realign on a pairhmm.Batch that has run a forward: (best haplotype per read, informative flags,
    AlignmentBatch of the reads against their best haplotypes)."""
    wl = batch.wl
    n = wl.n_reads
    prio = None
    if hap_priority is not None:
        prio = np.ascontiguousarray(hap_priority, dtype=np.float64)
        if len(prio) != wl.n_haps:
            raise ValueError("one priority per haplotype of the batch")
    cap = 2 * int(len(wl.bases)) + 4 * n
    res, off, start, length, ops = _result(n, cap)
    best = np.empty(max(n, 1), dtype=np.int32)
    inf = np.empty(max(n, 1), dtype=np.uint8)
    p = parameters.as_native()
    L, h = batch.engine.L, batch.engine.handle
    rc = L.ghmm_batch_realign(h, batch.h, prio.ctypes.data if prio is not None else None, ctypes.byref(p),
                              best.ctypes.data, inf.ctypes.data, ctypes.byref(res))
    native.check(rc, h)
    return best[:n], inf[:n].astype(bool), AlignmentBatch(off[:n], start[:n], length[:n], ops[:res.cigar_total])
