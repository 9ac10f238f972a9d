"""Pin the FP64 oracle against the reference's own golden vectors and known-answer tests (CPU).

Golden files (tests/golden, produced by make_golden.py from the reference test resources):
  hc_java_hmmresults.tsv       LOGLESS_CACHING dump, HaplotypeCallerIntegrationTest.java:2193-2243
                               (exact text match in the reference, so %e strings must match here)
  vector_pairhmm_testdata.tsv  VectorPairHMMUnitTest.java:30-106, tolerance 1e-5 (:100)
  hc_avx_hmmresults.tsv        the same pairs through GKL's FP32 AVX kernel
Known answers ported from PairHMMUnitTest.java and PairHMMModelUnitTest.java.
"""
import itertools
import math
import random

import numpy as np
import pytest

from conftest import load_golden
from oracle import oracle as O


def _eval(rows, f):
    return [f(h, r, q, i, d, g) for h, r, q, i, d, g, _ in rows]


def test_java_hmmresults_exact_text():
    rows = load_golden("hc_java_hmmresults.tsv")
    assert len(rows) == 284
    vals = _eval(rows, O.logless)
    mism = [(k, "%e" % v, rows[k][6]) for k, v in enumerate(vals) if "%e" % v != rows[k][6]]
    assert not mism, mism[:5]


def test_java_hmmresults_exact_log10_equals_logless():
    # expected.Exact.hmmresults.txt is byte-identical to the Java file: EXACT agrees with LOGLESS here
    rows = load_golden("hc_java_hmmresults.tsv")
    for h, r, q, i, d, g, _ in rows[:120]:
        a = O.logless(h, r, q, i, d, g)
        b = O.log10_hmm(h, r, q, i, d, g, exact=True)
        assert abs(a - b) < 1e-9


def test_vector_pairhmm_testdata_1e5():
    rows = load_golden("vector_pairhmm_testdata.tsv")
    assert len(rows) == 104
    vals = _eval(rows, O.logless)
    err = max(abs(v - float(row[6])) for v, row in zip(vals, rows))
    assert err <= 1e-5, err


def test_avx_golden_within_gkl_fp32_error():
    # GKL's FP32 results differ from FP64 by at most a few 1e-6 on these pairs
    rows = load_golden("hc_avx_hmmresults.tsv")
    vals = _eval(rows, O.logless)
    err = max(abs(v - float(row[6])) for v, row in zip(vals, rows))
    assert err <= 1e-5, err


# ---- PairHMMUnitTest known answers (no tristate correction, as the test's @BeforeClass sets) ----
CONTEXT = b"ACGTAATGACGATTGCA"
LEFT_FLANK = b"GATTTATCATCGAGTCTGC"
RIGHT_FLANK = b"CATGGATCGTTATCAGCTATCTCGAGGGATTCACTTAACAGTTTTA"
MASSIVE = 100


def _with_context(bases, left, right):
    return (LEFT_FLANK if left else b"") + CONTEXT + bases + CONTEXT + (RIGHT_FLANK if right else b"")


def _quals(n_read, read_len, q, gop, anchor):
    # PairHMMUnitTest.java:125-145 qualAsBytes
    if not anchor:
        return np.full(n_read, q, dtype=np.uint8)
    a = np.full(n_read, MASSIVE, dtype=np.uint8)
    if gop:
        a[len(CONTEXT)] = q
    else:
        a[len(CONTEXT):len(CONTEXT) + read_len] = q
    return a


def _basic_case(ref, read, bq, iq, dq, gcp, left, right, anchor):
    hap = _with_context(ref, left, right)
    rd = _with_context(read, False, False)
    n = len(rd)
    args = (hap, rd, _quals(n, len(read), bq, False, anchor), _quals(n, len(read), iq, True, anchor),
            _quals(n, len(read), dq, True, anchor), _quals(n, len(read), gcp, False, anchor))
    return hap, args


def _basic_cases(extensive=True):
    # PairHMMUnitTest.java:148-199 makeBasicLikelihoodTests
    base_quals = [10, 20, 30, 40, 50] if extensive else [30]
    indel_quals = [20, 30, 40, 50] if extensive else [40]
    gcps = [8, 10, 20] if extensive else [10]
    sizes = [2, 3, 4, 5, 7, 8, 9, 10, 20, 30, 35] if extensive else [2]
    for bq, iq, gcp in itertools.product(base_quals, indel_quals, gcps):
        for rb, db in itertools.product(b"ACGT", b"ACGT"):
            yield bytes([rb]), bytes([db]), bq, iq, gcp, (0 if rb == db else bq), False, False
        for size in sizes:
            for base in b"ACGT":
                exp = iq + (size - 2) * gcp
                for ins in (True, False):
                    small, big = bytes([base]), bytes([base]) * size
                    ref, read = (small, big) if ins else (big, small)
                    for left, right in ((False, False), (True, False), (False, True), (True, True)):
                        yield ref, read, bq, iq, gcp, exp, left, right


def test_basic_likelihoods_known_answers():
    # PairHMMUnitTest.java:239-256: |logless - theory| <= 0.2 and |logless - exact| <= 0.2,
    # |original - exact| <= 1e-3; we also check logless against exact much tighter.
    n = 0
    worst_exact = 0.0
    for ref, read, bq, iq, gcp, expq, left, right in _basic_cases(extensive=True):
        hap, args = _basic_case(ref, read, bq, iq, iq, gcp, left, right, anchor=True)
        expected = expq / -10.0 + 0.03 + math.log10(1.0 / len(hap))
        ll = O.logless(*args, tristate=False)
        ex = O.log10_hmm(*args, tristate=False, exact=True)
        orig = O.log10_hmm(*args, tristate=False, exact=False)
        assert abs(ll - expected) <= 0.2
        assert abs(ex - expected) <= 0.2
        assert abs(ll - ex) <= 0.2
        assert abs(orig - ex) <= 1e-3
        assert ll <= 0.0
        worst_exact = max(worst_exact, abs(ll - ex))
        n += 1
    assert n > 3000
    assert worst_exact < 1e-6


def test_optimized_likelihoods_random_vs_exact():
    # PairHMMUnitTest.java:201-237,258-270 (random sequences, sizes 3..160) -- sampled subset
    rnd = random.Random(1234)
    for _ in range(60):
        bq = rnd.choice([10, 30, 40, 60])
        iq = rnd.choice([20, 40, 60])
        gcp = rnd.choice([10, 20, 30])
        ref = bytes(rnd.choice(b"ACGT") for _ in range(rnd.choice([3, 20, 50, 90, 160])))
        read = bytes(rnd.choice(b"ACGT") for _ in range(rnd.choice([3, 20, 50, 90, 160])))
        hap, args = _basic_case(ref, read, bq, iq, iq, gcp, rnd.random() < 0.5, rnd.random() < 0.5, anchor=False)
        ll = O.logless(*args, tristate=False)
        ex = O.log10_hmm(*args, tristate=False, exact=True)
        assert abs(ll - ex) <= 1e-9 * max(1.0, abs(ex)) * 10


def _qual_to_prob(q):
    return 1.0 - 10 ** (q / -10.0)


@pytest.mark.parametrize("offset_both_sides", [True, False])
def test_mismatch_in_every_position(offset_both_sides):
    # PairHMMUnitTest.java:272-326
    hap = b"TTCTCTTCTGTTGTGGCTGGTT"
    match_q, mismatch_q, indel_q, offset = 90, 20, 80, 2
    n = len(hap) - (2 * offset if offset_both_sides else offset)
    for k in range(n):
        quals = np.full(n, match_q, dtype=np.uint8)
        quals[k] = mismatch_q
        mread = bytearray(hap[offset:offset + n])
        mread[k] = ord("T") if mread[k] == ord("C") else ord("C")
        gop = np.full(n, indel_q, dtype=np.uint8)
        res = O.logless(hap, bytes(mread), quals, gop, gop, gop, tristate=False)
        expected = math.log10(1.0 / len(hap) * _qual_to_prob(match_q) ** (n - 1) * 10 ** (mismatch_q / -10.0))
        assert abs(res - expected) <= 1e-2


def _expected_matching(read_len, ref_len, bq, iq):
    # PairHMMUnitTest.java:404-418
    init = abs(ref_len - read_len + 1) / ref_len
    if read_len < ref_len:
        return math.log10(init * _qual_to_prob(bq) ** read_len)
    if read_len > ref_len:
        return math.log10(init * _qual_to_prob(bq) ** ref_len * (10 ** (iq / -10.0)) ** (read_len - ref_len))
    return 0.0


@pytest.mark.parametrize("read_size,ref_size", [(r, h) for r in (1, 2, 5, 10) for h in (1, 2, 5, 10) if h > r])
def test_all_matching_read(read_size, ref_size):
    # PairHMMUnitTest.java:390-402 (tolerance 1e-3)
    read = b"A" * read_size
    ref = b"A" * ref_size
    q = lambda v: np.full(read_size, v, dtype=np.uint8)
    d = O.logless(ref, read, q(20), q(100), q(100), q(100), tristate=False)
    assert abs(d - _expected_matching(read_size, ref_size, 20, 100)) <= 1e-3


@pytest.mark.parametrize("read_size,ref_size", [(r, h) for r in (1, 2, 5, 10) for h in (1, 2, 5, 10) if h > r])
def test_multiple_read_matches_in_haplotype(read_size, ref_size):
    # PairHMMUnitTest.java:341-360
    read = b"A" * read_size
    ref = b"CC" + b"A" * ref_size + b"GGA"
    q = lambda v: np.full(read_size, v, dtype=np.uint8)
    assert O.logless(ref, read, q(20), q(37), q(37), q(10), tristate=False) <= 0.0


def test_really_big_reads():
    # PairHMMUnitTest.java:420-457 (no exception, valid result) -- the largest combination
    read = b"ACCAAGTAGTCACCGT" * 50
    ref = b"ACCAAGTAGTCACCGTAACG" * 100
    q = lambda v: np.full(len(read), v, dtype=np.uint8)
    v = O.logless(ref, read, q(30), q(40), q(40), q(10), tristate=False)
    assert v <= 0.0 and math.isfinite(v)


def test_trans_probs_match_model_definition():
    # PairHMMModelUnitTest.java:19-112: qualToTransProbs vs the model's definition (1e-9)
    for ins, dl, gcp in [(10, 10, 10), (30, 45, 10), (45, 45, 10), (1, 100, 20), (127, 0, 127), (0, 0, 0)]:
        t = O.trans_probs(ins, dl, gcp)
        e = lambda q: 10 ** (q / -10.0)
        assert abs(t[2] - e(ins)) < 1e-12  # MI
        assert abs(t[4] - e(dl)) < 1e-12  # MD
        assert abs(t[1] - (1 - e(gcp))) < 1e-12  # IM
        assert t[3] == t[5] == pytest.approx(e(gcp), abs=1e-15)
        # matchToMatch = 1 - (e(ins) + e(del)) up to the Jacobian table step (1e-4 in log10)
        assert abs(t[0] - (1 - min(1.0, e(ins) + e(dl)))) < 3e-4 * (e(ins) + e(dl)) + 1e-12
        tl = O.trans_probs(ins, dl, gcp, log10=True)
        assert abs(tl[2] - (-0.1 * ins)) < 1e-12 and abs(tl[4] - (-0.1 * dl)) < 1e-12
        if t[0] > 0:
            assert abs(10 ** tl[0] - t[0]) < 1e-9


def test_jacobian_table_size_and_ends():
    L = O.lib()
    assert L.oracle_jacobian_size() == 80001
    assert abs(L.oracle_jacobian_value(0) - math.log10(2.0)) < 1e-15
    assert L.oracle_jacobian_value(80000) < 1e-8


def test_empty_read_and_haplotype_give_minus_infinity():
    # LoglessPairHMM.java:62-67 with paddedReadLength == 1: the sum is 0 -> -Infinity
    assert O.logless(b"ACGT", b"", [], [], [], []) == -math.inf
    assert O.logless(b"", b"A", [30], [45], [45], [10]) == -math.inf


def test_n_matches_everything():
    # LoglessPairHMM.java:89: x == y || x == 'N' || y == 'N' -> match prior
    q, g, c = [30], [45], [10]
    a = O.logless(b"A", b"A", q, g, g, c)
    assert O.logless(b"N", b"A", q, g, g, c) == a
    assert O.logless(b"A", b"N", q, g, g, c) == a
    assert O.logless(b"C", b"A", q, g, g, c) < a
    # an N column matches every shifted alignment too, so it can only raise the likelihood
    q5, g5, c5 = [30] * 5, [45] * 5, [10] * 5
    assert O.logless(b"ANGTA", b"ACGTA", q5, g5, g5, c5) >= O.logless(b"ACGTA", b"ACGTA", q5, g5, g5, c5)


def test_validate_rejects_out_of_range():
    L = O.lib()
    ok = np.array([30, 254], dtype=np.uint8)
    bad_q = np.array([30, 255], dtype=np.uint8)
    pen = np.array([45, 127], dtype=np.uint8)
    bad_pen = np.array([45, 128], dtype=np.uint8)
    p = lambda a: a.ctypes.data_as(O._u8p)
    assert L.oracle_validate_read(p(ok), p(pen), p(pen), p(pen), 2) == 0
    assert L.oracle_validate_read(p(bad_q), p(pen), p(pen), p(pen), 2) == -1
    assert L.oracle_validate_read(p(ok), p(bad_pen), p(pen), p(pen), 2) == -1
