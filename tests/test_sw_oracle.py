"""The Smith-Waterman oracle, pinned to the reference's own known answers: the cases of
SmithWatermanAlignerAbstractUnitTest (every SmithWatermanAligner implementation runs them), transcribed by
tests/golden/make_sw_golden.py into sw_unit_cases.json, plus its flank-length property test.  The C restatement
(oracle/sw_oracle.c, also the timed CPU baseline) must agree with the Python one everywhere."""
import json
import os
import random

import pytest

from conftest import GOLDEN
from oracle import oracle as O
from oracle import postprocess as P
from oracle import smithwaterman as S

CASES = json.load(open(os.path.join(GOLDEN, "sw_unit_cases.json")))


def _ops_to_elems(ops):
    return [(o & 15, o >> 4) for o in ops]


@pytest.mark.parametrize("case", CASES["cases"], ids=lambda c: f"{c['name']}-{c['strategy']}")
def test_python_oracle_reproduces_the_reference_known_answers(case):
    elems, off = S.align(case["ref"].encode(), case["alt"].encode(), case["params"], S.STRATEGIES[case["strategy"]])
    assert S.cigar_string(elems) == case["cigar"]
    assert off == case["offset"]


@pytest.mark.parametrize("case", CASES["cases"], ids=lambda c: f"{c['name']}-{c['strategy']}")
def test_c_oracle_reproduces_the_reference_known_answers(case):
    ops, off = O.sw_align(case["ref"].encode(), case["alt"].encode(), case["params"], S.STRATEGIES[case["strategy"]])
    assert S.cigar_string(_ops_to_elems(ops)) == case["cigar"]
    assert off == case["offset"]


def _flank_pair(f, padded: bool):
    ref = f["paddedRef"] if padded else f["notPaddedRef"]
    hap = f["paddedHap"] if padded else f["notPaddedHap"]
    return (f["pad"] + ref + f["pad"]).encode(), (f["pad"] + hap + f["pad"]).encode()


def test_identical_alignments_with_differing_flank_lengths():
    # testForIdenticalAlignmentsWithDifferingFlankLengths: the indel elements do not depend on the flanks
    f = CASES["flank_test"]
    a = S.align(*_flank_pair(f, True), f["params"], S.SOFTCLIP)[0]
    b = S.align(*_flank_pair(f, False), f["params"], S.SOFTCLIP)[0]
    assert len(a) == len(b)
    for (op1, n1), (op2, n2) in zip(a, b):
        if op1 == S.OP_M and op2 == S.OP_M:
            continue
        assert (op1, n1) == (op2, n2)


def test_empty_sequences_are_rejected():
    with pytest.raises(ValueError, match="non-empty sequences"):
        S.align(b"", b"A")
    with pytest.raises(ValueError, match="non-empty sequences"):
        S.align(b"A", b"")
    with pytest.raises(ValueError):
        O.sw_align(b"", b"A", S.ORIGINAL_DEFAULT, S.SOFTCLIP)


def _random_pair(rng):
    n, m = rng.randint(1, 45), rng.randint(1, 45)
    alph = rng.choice([b"AC", b"ACGT", b"ACGTN"])
    ref = bytes(rng.choice(alph) for _ in range(n))
    if rng.random() < 0.5 and n > 3:
        a = rng.randint(0, n - 1)
        alt = bytearray(ref[a:rng.randint(a + 1, n)])
        for k in range(len(alt)):
            if rng.random() < 0.1:
                alt[k] = rng.choice(alph)
        return ref, bytes(alt)
    return ref, bytes(rng.choice(alph) for _ in range(m))


def test_c_oracle_equals_python_oracle_on_random_pairs():
    rng = random.Random(7)
    sets = [S.ORIGINAL_DEFAULT, S.STANDARD_NGS, S.NEW_SW_PARAMETERS, S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS]
    for _ in range(1500):
        ref, alt = _random_pair(rng)
        params = rng.choice(sets + [(rng.randint(0, 6), rng.randint(-6, 0), rng.randint(-9, 0), rng.randint(-4, 0))])
        st, sc = rng.randint(0, 3), rng.random() < 0.5
        e, o = S.align(ref, alt, params, st, sc)
        ops, off = O.sw_align(ref, alt, params, st, sc)
        assert (_ops_to_elems(ops), off) == (e, o), (ref, alt, params, st, sc)


def test_java_int_wraparound_is_reproduced():
    # parameters near the int range: Java's adds wrap at 32 bits, and so do both restatements
    params = (2 ** 30, -(2 ** 30), -(2 ** 31) + 5, -(2 ** 30))
    rng = random.Random(3)
    for _ in range(200):
        ref, alt = _random_pair(rng)
        st = rng.randint(0, 3)
        e, o = S.align(ref, alt, params, st, False)
        ops, off = O.sw_align(ref, alt, params, st, False)
        assert (_ops_to_elems(ops), off) == (e, o)


def test_batch_oracle_equals_single_calls():
    rng = random.Random(9)
    pairs = [_random_pair(rng) for _ in range(300)]
    refs, alts = [p[0] for p in pairs], [p[1] for p in pairs]
    ref_off = [0]
    alt_off = [0]
    for r, a in pairs:
        ref_off.append(ref_off[-1] + len(r))
        alt_off.append(alt_off[-1] + len(a))
    ops, start, n_ops, off = O.sw_align_pairs(b"".join(refs), ref_off[:-1], [len(r) for r in refs], b"".join(alts),
                                              alt_off[:-1], [len(a) for a in alts], S.ORIGINAL_DEFAULT, S.SOFTCLIP)
    for i, (r, a) in enumerate(pairs):
        e, o = S.align(r, a, S.ORIGINAL_DEFAULT, S.SOFTCLIP)
        assert _ops_to_elems(ops[start[i]:start[i] + n_ops[i]]) == e and off[i] == o


def test_best_allele_breaking_ties():
    # the unique best wins when it leads by more than the informative threshold
    assert P.best_allele_breaking_ties([-5.0, -1.0, -3.0], [1.0, 0.0, 0.0]) == (1, True)
    # within the threshold the priority decides: the reference haplotype (priority 1) takes the read
    assert P.best_allele_breaking_ties([-1.1, -1.0, -3.0], [1.0, 0.0, 0.0]) == (0, False)
    # without priorities the likelihood decides, and the read is not informative
    assert P.best_allele_breaking_ties([-1.1, -1.0, -3.0], None) == (1, False)
    # equal priorities keep the likelihood order
    assert P.best_allele_breaking_ties([-1.1, -1.0, -3.0], [0.0, 0.0, 0.0]) == (1, False)
    # a single haplotype is informative (its second best is -inf)
    assert P.best_allele_breaking_ties([-2.0], [0.0]) == (0, True)
    assert P.best_allele_breaking_ties([], None) == (-1, False)
