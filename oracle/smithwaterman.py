"""CPU restatement of GATK's Smith-Waterman aligner (test infrastructure: the oracle for ghmm_sw_align and
ghmm_sw_align_batch).  Pure Python loops, for small cases; oracle/sw_oracle.c is the same algorithm in C for
larger ones.  Follows (paths inside the GATK repository, src/main/java/org/broadinstitute/hellbender/):

  SmithWatermanJavaAligner.align            utils/smithwaterman/SmithWatermanJavaAligner.java:59-98
  SmithWatermanJavaAligner.calculateMatrix  :109-228  (Gotoh-style best-gap tracking with gap lengths)
  SmithWatermanJavaAligner.calculateCigar   :261-379  (end-cell choice per overhang strategy, traceback)
  SWNativeAlignerWrapper.align               utils/smithwaterman/SWNativeAlignerWrapper.java:31-59
      (exact-substring shortcut for SOFTCLIP and IGNORE; the native aligner itself has none)
  Utils.lastIndexOf                          utils/Utils.java:1124-1138
  SWParameters(match, mismatch, gap open, gap extend) and SWOverhangStrategy {SOFTCLIP, INDEL, LEADING_INDEL,
  IGNORE} come from gatk-native-bindings 1.1.0 (not vendored): plain holders, no arithmetic of their own.

Java int arithmetic wraps at 32 bits; every sum here goes through _i32 so that results match for any
parameter values.
"""
from __future__ import annotations

SOFTCLIP, INDEL, LEADING_INDEL, IGNORE = 0, 1, 2, 3
STRATEGIES = {"SOFTCLIP": SOFTCLIP, "INDEL": INDEL, "LEADING_INDEL": LEADING_INDEL, "IGNORE": IGNORE}

# SmithWatermanAlignmentConstants.java:30,38,52,68
ORIGINAL_DEFAULT = (3, -1, -4, -3)
STANDARD_NGS = (25, -50, -110, -6)
NEW_SW_PARAMETERS = (200, -150, -260, -11)
ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS = (10, -15, -30, -5)

MATRIX_MIN_CUTOFF = -100000000        # (int) -1.0e8
LOW_INIT_VALUE = -(2 ** 31) // 2      # Integer.MIN_VALUE / 2

# htsjdk CigarOperator BAM codes of the four operators the aligner emits
OP_M, OP_I, OP_D, OP_S = 0, 1, 2, 4
OP_CHARS = "MIDNSHP=X"


def _i32(v: int) -> int:
    v &= 0xFFFFFFFF
    return v - (1 << 32) if v & 0x80000000 else v


def last_index_of(reference: bytes, query: bytes) -> int:
    """Utils.lastIndexOf: the rightmost start of query inside reference, or -1."""
    n, m = len(reference), len(query)
    for r in range(n - m, -1, -1):
        if reference[r:r + m] == query:
            return r
    return -1


def calculate_matrix(reference: bytes, alternate: bytes, params, strategy: int):
    """The score matrix sw[n+1][m+1] and the backtrack matrix (0 diagonal, -k horizontal gap of k, +k vertical)."""
    w_match, w_mismatch, w_open, w_extend = params
    n, m = len(reference) + 1, len(alternate) + 1
    sw = [[0] * m for _ in range(n)]
    btrack = [[0] * m for _ in range(n)]
    best_gap_v = [LOW_INIT_VALUE] * (m + 1)
    gap_size_v = [0] * (m + 1)
    best_gap_h = [LOW_INIT_VALUE] * (n + 1)
    gap_size_h = [0] * (n + 1)
    if strategy in (INDEL, LEADING_INDEL):
        top = sw[0]
        top[1] = w_open
        cur = w_open
        for j in range(2, m):
            cur = _i32(cur + w_extend)
            top[j] = cur
        sw[1][0] = w_open
        cur = w_open
        for i in range(2, n):
            cur = _i32(cur + w_extend)
            sw[i][0] = cur
    for i in range(1, n):
        a = reference[i - 1]
        last, cur_row, bt = sw[i - 1], sw[i], btrack[i]
        for j in range(1, m):
            step_diag = _i32(last[j - 1] + (w_match if a == alternate[j - 1] else w_mismatch))
            prev_gap = _i32(last[j] + w_open)
            best_gap_v[j] = _i32(best_gap_v[j] + w_extend)
            if prev_gap > best_gap_v[j]:
                best_gap_v[j] = prev_gap
                gap_size_v[j] = 1
            else:
                gap_size_v[j] += 1
            step_down, kd = best_gap_v[j], gap_size_v[j]
            prev_gap = _i32(cur_row[j - 1] + w_open)
            best_gap_h[i] = _i32(best_gap_h[i] + w_extend)
            if prev_gap > best_gap_h[i]:
                best_gap_h[i] = prev_gap
                gap_size_h[i] = 1
            else:
                gap_size_h[i] += 1
            step_right, ki = best_gap_h[i], gap_size_h[i]
            if step_diag >= step_down and step_diag >= step_right:
                cur_row[j] = max(MATRIX_MIN_CUTOFF, step_diag)
                bt[j] = 0
            elif step_right >= step_down:
                cur_row[j] = max(MATRIX_MIN_CUTOFF, step_right)
                bt[j] = -ki
            else:
                cur_row[j] = max(MATRIX_MIN_CUTOFF, step_down)
                bt[j] = kd
    return sw, btrack


def _push(elems, op: int, length: int):
    elems.append((op, length))


def calculate_cigar(sw, btrack, strategy: int):
    """(cigar elements [(op, length)], alignment offset) from the matrices, as calculateCigar builds them."""
    ref_len, alt_len = len(sw) - 1, len(sw[0]) - 1
    p1 = p2 = 0
    maxscore = -(2 ** 31)
    segment_length = 0
    if strategy == INDEL:
        p1, p2 = ref_len, alt_len
    else:
        p2 = alt_len
        for i in range(1, len(sw)):
            if sw[i][alt_len] >= maxscore:
                p1, maxscore = i, sw[i][alt_len]
        if strategy != LEADING_INDEL:
            bottom = sw[ref_len]
            for j in range(1, len(bottom)):
                s = bottom[j]
                if s > maxscore or (s == maxscore and abs(ref_len - j) < abs(p1 - p2)):
                    p1, p2, maxscore = ref_len, j, s
                    segment_length = alt_len - j
    lce = []
    if segment_length > 0 and strategy == SOFTCLIP:
        _push(lce, OP_S, segment_length)
        segment_length = 0
    state = OP_M
    while True:
        btr = btrack[p1][p2]
        step = 1
        if btr > 0:
            new_state, step = OP_D, btr
        elif btr < 0:
            new_state, step = OP_I, -btr
        else:
            new_state = OP_M
        if new_state == OP_M:
            p1 -= 1
            p2 -= 1
        elif new_state == OP_I:
            p2 -= step
        else:
            p1 -= step
        if new_state == state:
            segment_length += step
        else:
            if segment_length > 0:
                _push(lce, state, segment_length)
            segment_length = step
            state = new_state
        if not (p1 > 0 and p2 > 0):
            break
    if strategy == SOFTCLIP:
        _push(lce, state, segment_length)
        if p2 > 0:
            _push(lce, OP_S, p2)
        offset = p1
    elif strategy == IGNORE:
        _push(lce, state, segment_length + p2)
        offset = p1 - p2
    else:
        _push(lce, state, segment_length)
        if p1 > 0:
            _push(lce, OP_D, p1)
        elif p2 > 0:
            _push(lce, OP_I, p2)
        offset = 0
    lce.reverse()
    return lce, offset


def align(reference: bytes, alternate: bytes, params=ORIGINAL_DEFAULT, strategy: int = SOFTCLIP,
          shortcut: bool = True):
    """SmithWatermanJavaAligner.align (shortcut=True) or the native binding's align (shortcut=False, the
    wrapper having found no exact match): (cigar elements, alignment offset)."""
    reference, alternate = bytes(reference), bytes(alternate)
    if not reference or not alternate:
        raise ValueError("Non-null, non-empty sequences are required for the Smith-Waterman calculation")
    if strategy not in (SOFTCLIP, INDEL, LEADING_INDEL, IGNORE):
        raise ValueError(f"unknown overhang strategy {strategy}")
    if shortcut and strategy in (SOFTCLIP, IGNORE):
        idx = last_index_of(reference, alternate)
        if idx != -1:
            return [(OP_M, len(alternate))], idx
    sw, bt = calculate_matrix(reference, alternate, params, strategy)
    return calculate_cigar(sw, bt, strategy)


def cigar_string(elems) -> str:
    """htsjdk Cigar.toString of the elements (an empty cigar prints as '*'); consecutive elements with the same
    operator stay separate, as the aligner builds the Cigar from its element list directly."""
    if not elems:
        return "*"
    return "".join(f"{n}{OP_CHARS[op]}" for op, n in elems)
