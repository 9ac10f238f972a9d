"""CPU restatement of the read preparation before the PairHMM (test infrastructure; the oracle for
ghmm_compute_regions_raw).  Pure Python loops, for small cases.  Follows (paths inside the GATK repository):

  PairHMMLikelihoodCalculationEngine.modifyReadQualities / capMinimumReadQualities / setToFixedValueIfTooLow
      src/main/java/org/broadinstitute/hellbender/tools/walkers/haplotypecaller/
      PairHMMLikelihoodCalculationEngine.java:283-322
  PCR indel error model: initializePCRErrorModel, getErrorModelAdjustedQual, applyPCRErrorModel     :331-371
      (MIN_ADJUSTED_QSCORE 10 :32, INITIAL_QSCORE 40.0 :35, PCRErrorModel rate factors :53-71)
  ReadLikelihoodCalculationEngine.findTandemRepeatUnits (MAX_STR_UNIT_LENGTH 8, MAX_REPEAT_LENGTH 20)
      ReadLikelihoodCalculationEngine.java:25-26,193-253
  GATKVariantContextUtils.findNumberOfRepetitions   utils/variant/GATKVariantContextUtils.java:949-1011
  MathUtils.fastRound                               utils/MathUtils.java:428-430
  ReadUtils.getBaseInsertionQualities / getBaseDeletionQualities (default 45)   utils/read/ReadUtils.java:44,838-862
  StandardPairHMMInputScoreImputator (constant gap continuation penalty)
  DragstrPairHMMInputScoreImputator.impute (MAX_GOP_IN_READ 40, 45 / 10 at the last base)
      tools/walkers/haplotypecaller/DragstrPairHMMInputScoreImputator.java:22-31,54-88
  DragstrReadSTRAnalyzer (repeat count per period and position, most repeated period with ties to the shorter one)
      utils/pairhmm/DragstrReadSTRAnalyzer.java:110-139; the position-by-position definition its test checks against,
      DragstrReadSTRAnalyzerTest.calculateExpectedRepeatLength (src/test/.../DragstrReadSTRAnalyzerTest.java:131-168)
  DragstrParams.lookup (periods / repeats past the table use its last row / column)
      utils/dragstr/DragstrParams.java:194-220
"""
from __future__ import annotations

import math

MAX_STR_UNIT_LENGTH = 8
MAX_REPEAT_LENGTH = 20
MIN_USABLE_Q_SCORE = 6
MIN_ADJUSTED_QSCORE = 10
INITIAL_QSCORE = 40.0
DEFAULT_INDEL_QUAL = 45


def fast_round(d: float) -> int:
    return int(d + 0.5) if d > 0.0 else int(d - 0.5)


def pcr_cache(rate_factor: float) -> list[int]:
    """getErrorModelAdjustedQual for repeat lengths 0..MAX_REPEAT_LENGTH (a Java byte: values fit in 0..40)."""
    return [max(MIN_ADJUSTED_QSCORE, fast_round(INITIAL_QSCORE - math.exp(rl / (rate_factor * math.pi)) + 1.0))
            for rl in range(MAX_REPEAT_LENGTH + 1)]


def repetitions(unit: bytes, test: bytes, leading: bool) -> int:
    """findNumberOfRepetitions: how many copies of unit the test string starts (leading) or ends (trailing) with."""
    n, L = len(test), len(unit)
    if n == 0:
        return 0
    count = 0
    starts = range(0, n - L + 1, L) if leading else range(n - L, -1, -L)
    for s in starts:
        if test[s:s + L] == unit:
            count += 1
        else:
            return count
    return count


def tandem_repeat_length(b: bytes, offset: int) -> int:
    """findTandemRepeatUnits(...).getRight(): the repeat count around offset, capped at MAX_REPEAT_LENGTH."""
    max_bw = 0
    bw_unit = b[offset:offset + 1]
    for str_len in range(1, MAX_STR_UNIT_LENGTH + 1):
        if offset + 1 - str_len < 0:
            break
        max_bw = repetitions(b[offset - str_len + 1:offset + 1], b[0:offset + 1], False)
        if max_bw > 1:
            bw_unit = b[offset - str_len + 1:offset + 1]
            break
    max_rl = max_bw
    if offset < len(b) - 1:
        fw_unit = b[offset + 1:offset + 2]
        max_fw = 0
        for str_len in range(1, MAX_STR_UNIT_LENGTH + 1):
            if offset + str_len + 1 > len(b):
                break
            max_fw = repetitions(b[offset + 1:offset + str_len + 1], b[offset + 1:], True)
            if max_fw > 1:
                fw_unit = b[offset + 1:offset + str_len + 1]
                break
        if fw_unit == bw_unit:
            max_rl = max_bw + max_fw
        else:
            max_rl = max_fw + repetitions(fw_unit, b[0:offset + 1], False)
    return min(max_rl, MAX_REPEAT_LENGTH)


def str_repeats(seq: bytes, pos: int, period: int) -> int:
    """Repeat count of `period` at `pos`: the longest tandem run (in units) of a period-mer that contains pos or
    starts right after it; a unit starting at 0 counts one fewer (not below 1) for positions before period - 1."""
    n = len(seq)
    if period > n:
        return 0
    best = 0
    start = max(0, pos - period + 1)
    while start <= pos + 1 and start + period <= n:
        unit = seq[start:start + period]
        count = 1
        off = start + period
        while off + period <= n and seq[off:off + period] == unit:
            count += 1
            off += period
        off = start - period
        while off >= 0 and seq[off:off + period] == unit:
            count += 1
            off -= period
        if pos < period - 1 and start == 0:
            count = max(1, count - 1)
        best = max(best, count)
        start += 1
    return best


def str_analyze(seq: bytes, max_period: int):
    """(most repeated period, its repeat count) per position; ties go to the shorter period."""
    periods, repeats = [], []
    for pos in range(len(seq)):
        bp, br = 1, str_repeats(seq, pos, 1)
        for p in range(2, max_period + 1):
            r = str_repeats(seq, pos, p)
            if r > br:
                bp, br = p, r
        periods.append(bp)
        repeats.append(br)
    return periods, repeats


def java_round(x: float) -> int:
    """Math.round(double): half up."""
    r = math.floor(x)
    return int(r + 1 if x - r >= 0.5 else r)


def dragstr_impute(bases, gop_table, gcp_table):
    """DragstrPairHMMInputScoreImputator.impute: (GOP plane, GCP plane) of one read, tables [max_period][max_repeats]
    (DragstrParams.gop / gcp at [period - 1][repeats - 1])."""
    b = bytes(bases)
    n = len(b)
    max_period, max_repeats = len(gop_table), len(gop_table[0])
    gop, gcp = bytearray(n), bytearray(n)
    if n == 0:
        return bytes(gop), bytes(gcp)
    periods, repeats = str_analyze(b, max_period)
    for i in range(n - 1):
        p, r = periods[i], repeats[i]
        pi = p - 1 if p < max_period else max_period - 1
        ri = r - 1 if r < max_repeats else max_repeats - 1
        gop[i] = java_round(min(40.0, float(gop_table[pi][ri]))) & 0xFF
        gcp[i] = java_round(float(gcp_table[pi][ri])) & 0xFF
    gop[n - 1], gcp[n - 1] = 45, 10
    return bytes(gop), bytes(gcp)


def prepare_read(bases, quals, ins, dels, mapq: int, threshold: int = 18, cap_to_mapq: bool = True,
                 rate_factor: float = 0.0, gcp: int = 10, dragstr=None):
    """The five PairHMM inputs of one read: (bases, quals, insertion GOP, deletion GOP, GCP).  With dragstr = (gop,
    gcp) tables the DRAGstr imputation gives the three gap planes (PairHMM.computeLog10Likelihoods takes them from
    the imputator, not from the read's capped BI / BD values)."""
    b = bytes(bases)
    n = len(b)
    q = [int(x) for x in quals]
    if dragstr is not None:
        signed = lambda v: v - 256 if v > 127 else v
        for i in range(n):
            if cap_to_mapq:
                q[i] = min(q[i], mapq) & 0xFF
            q[i] = MIN_USABLE_Q_SCORE if signed(q[i]) < threshold else q[i]
        g, c = dragstr_impute(b, dragstr[0], dragstr[1])
        return b, bytes(q), g, g, c
    i_q = [DEFAULT_INDEL_QUAL] * n if ins is None else [int(x) for x in ins]
    d_q = [DEFAULT_INDEL_QUAL] * n if dels is None else [int(x) for x in dels]
    if rate_factor != 0.0:  # applyPCRErrorModel
        cache = pcr_cache(rate_factor)
        for i in range(1, n):
            rl = tandem_repeat_length(b, i - 1)
            i_q[i - 1] = min(i_q[i - 1], cache[rl])
            d_q[i - 1] = min(d_q[i - 1], cache[rl])
    signed = lambda v: v - 256 if v > 127 else v  # setToFixedValueIfTooLow compares Java (signed) bytes
    for i in range(n):  # capMinimumReadQualities
        if cap_to_mapq:
            q[i] = min(q[i], mapq) & 0xFF
        q[i] = MIN_USABLE_Q_SCORE if signed(q[i]) < threshold else q[i]
        i_q[i] = MIN_USABLE_Q_SCORE if signed(i_q[i]) < MIN_USABLE_Q_SCORE else i_q[i]
        d_q[i] = MIN_USABLE_Q_SCORE if signed(d_q[i]) < MIN_USABLE_Q_SCORE else d_q[i]
    return b, bytes(q), bytes(i_q), bytes(d_q), bytes([gcp] * n)
