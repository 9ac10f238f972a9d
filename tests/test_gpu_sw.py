"""Smith-Waterman on the GPU (ghmm_sw_align, ghmm_sw_align_batch, ghmm_batch_realign) against the oracle: the
reference's own known answers, random pairs of every strategy and parameter set against oracle/sw_oracle.c, alts
long enough to run in several strips, several passes over a small traceback buffer, Java's int wraparound, and the
read-to-best-haplotype realignment of a PairHMM batch.  Cigars and offsets must be identical."""
import json
import os
import random

import numpy as np
import pytest

from conftest import GOLDEN
from gatk_gb300 import native
from gatk_gb300 import smithwaterman as SWG
from gatk_gb300 import workload as W
from oracle import oracle as O
from oracle import postprocess as P
from oracle import smithwaterman as S

pytestmark = pytest.mark.gpu

CASES = json.load(open(os.path.join(GOLDEN, "sw_unit_cases.json")))


@pytest.fixture(scope="module")
def aligner():
    a = SWG.SmithWatermanCudaAligner()
    yield a
    a.close()


def _params(p):
    return SWG.SWParameters(*p)


@pytest.mark.parametrize("case", CASES["cases"], ids=lambda c: f"{c['name']}-{c['strategy']}")
def test_known_answers_through_the_wrapper(aligner, case):
    a = aligner.align(case["ref"].encode(), case["alt"].encode(), _params(case["params"]),
                      SWG.SWOverhangStrategy[case["strategy"]])
    assert (a.get_cigar(), a.get_alignment_offset()) == (case["cigar"], case["offset"])


@pytest.mark.parametrize("case", CASES["cases"], ids=lambda c: f"{c['name']}-{c['strategy']}")
def test_known_answers_through_the_native_binding(aligner, case):
    # the binding itself has no shortcut: these substring cases run the full recurrence on the device
    ref, alt, st = case["ref"].encode(), case["alt"].encode(), S.STRATEGIES[case["strategy"]]
    a = aligner.align_native(ref, alt, _params(case["params"]), SWG.SWOverhangStrategy(st))
    e, o = S.align(ref, alt, case["params"], st, shortcut=False)
    assert (a.get_cigar(), a.get_alignment_offset()) == (S.cigar_string(e), o)


def test_flank_lengths_do_not_move_the_indels(aligner):
    f = CASES["flank_test"]
    pad = f["pad"]
    res = []
    for ref, hap in ((f["paddedRef"], f["paddedHap"]), (f["notPaddedRef"], f["notPaddedHap"])):
        b = aligner.align_many([(pad + ref + pad).encode()], [(pad + hap + pad).encode()], _params(f["params"]),
                               SWG.SWOverhangStrategy.SOFTCLIP)
        res.append([(int(o) & 15, int(o) >> 4) for o in b.ops(0)])
    a, b = res
    assert len(a) == len(b)
    for (op1, n1), (op2, n2) in zip(a, b):
        if op1 == op2 == S.OP_M:
            continue
        assert (op1, n1) == (op2, n2)


def _mutate(rng, seq: bytes, alph: bytes, sub: float, indel: float) -> bytes:
    out = bytearray()
    for c in seq:
        u = rng.random()
        if u < indel / 2:
            continue
        if u < indel:
            out.append(rng.choice(alph))
        out.append(rng.choice(alph) if rng.random() < sub else c)
    return bytes(out) or seq[:1]


def _pairs(rng, n, ref_len, alt_len, alph=b"ACGT"):
    refs, alts = [], []
    for _ in range(n):
        r = bytes(rng.choice(alph) for _ in range(rng.randint(*ref_len)))
        m = rng.randint(*alt_len)
        u = rng.random()
        if u < 0.6 and len(r) > 2:
            a0 = rng.randint(0, max(0, len(r) - m))
            a = _mutate(rng, r[a0:a0 + m], alph, 0.03, 0.01)
        elif u < 0.7 and len(r) > 2:
            a0 = rng.randint(0, len(r) - 1)
            a = r[a0:a0 + m]  # exact substring: the shortcut's case
        else:
            a = bytes(rng.choice(alph) for _ in range(m))
        refs.append(r)
        alts.append(a)
    return refs, alts


def _oracle_many(refs, alts, params, strategy, shortcut):
    ref_off = np.cumsum([0] + [len(r) for r in refs])[:-1]
    alt_off = np.cumsum([0] + [len(a) for a in alts])[:-1]
    ops, start, n_ops, off = O.sw_align_pairs(b"".join(refs), ref_off, [len(r) for r in refs], b"".join(alts),
                                              alt_off, [len(a) for a in alts], params, strategy, shortcut)
    return ops, start, n_ops, off


def _assert_same(got: SWG.AlignmentBatch, refs, alts, params, strategy, shortcut):
    ops, start, n_ops, off = _oracle_many(refs, alts, params, strategy, shortcut)
    np.testing.assert_array_equal(got.offset, off)
    np.testing.assert_array_equal(got.cigar_len, n_ops)
    for i in range(len(refs)):
        np.testing.assert_array_equal(got.ops(i), ops[start[i]:start[i] + n_ops[i]], err_msg=f"pair {i}")


PARAM_SETS = [S.ORIGINAL_DEFAULT, S.STANDARD_NGS, S.NEW_SW_PARAMETERS, S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS]


@pytest.mark.parametrize("strategy", [S.SOFTCLIP, S.INDEL, S.LEADING_INDEL, S.IGNORE])
@pytest.mark.parametrize("params", PARAM_SETS, ids=["original", "standard_ngs", "new_sw", "best_haplotype"])
def test_random_pairs_match_the_oracle(aligner, strategy, params):
    rng = random.Random(hash((strategy, params)) & 0xFFFF)
    refs, alts = _pairs(rng, 300, (1, 420), (1, 300))
    for shortcut in (True, False):
        got = aligner.align_many(refs, alts, SWG.SWParameters(*params), SWG.SWOverhangStrategy(strategy), shortcut)
        _assert_same(got, refs, alts, params, strategy, shortcut)


def test_every_alt_width_and_several_strips(aligner):
    # alts of 1..8 lanes' worth of columns (K = 1..8) and alts of 2-5 strips of 256 columns
    rng = random.Random(21)
    refs, alts = [], []
    for m in list(range(1, 260, 7)) + [256, 257, 511, 512, 513, 700, 1100]:
        for _ in range(2):
            a = bytes(rng.choice(b"ACGT") for _ in range(m))
            flank = lambda: bytes(rng.choice(b"ACGT") for _ in range(rng.randint(0, 150)))
            r = flank() + _mutate(rng, a, b"ACGT", 0.03, 0.01) + flank()
            refs.append(r)
            alts.append(a)
    assert max(len(a) for a in alts) == 1100
    for st in (S.SOFTCLIP, S.INDEL):
        got = aligner.align_many(refs, alts, SWG.ORIGINAL_DEFAULT, SWG.SWOverhangStrategy(st), False)
        _assert_same(got, refs, alts, S.ORIGINAL_DEFAULT, st, False)


def test_small_alphabets_and_unusual_bytes(aligner):
    # long runs of equal scores stress the tie rules; N and lower-case bytes compare as raw bytes like Java's
    rng = random.Random(5)
    for alph in (b"A", b"AC", b"ACGTN", b"acgtACGT"):
        refs, alts = _pairs(rng, 150, (1, 120), (1, 90), alph)
        for st in (S.SOFTCLIP, S.LEADING_INDEL, S.IGNORE):
            got = aligner.align_many(refs, alts, SWG.STANDARD_NGS, SWG.SWOverhangStrategy(st), True)
            _assert_same(got, refs, alts, S.STANDARD_NGS, st, True)


def test_java_int_wraparound(aligner):
    params = (2 ** 30, -(2 ** 30), -(2 ** 31) + 5, -(2 ** 30))
    rng = random.Random(8)
    refs, alts = _pairs(rng, 120, (1, 60), (1, 60))
    for st in range(4):
        got = aligner.align_many(refs, alts, SWG.SWParameters(*params), SWG.SWOverhangStrategy(st), False)
        _assert_same(got, refs, alts, params, st, False)


def test_several_passes_over_a_small_traceback_buffer():
    rng = random.Random(12)
    refs, alts = _pairs(rng, 400, (200, 600), (100, 250))
    with SWG.SmithWatermanCudaAligner() as a:
        a.set_traceback_budget(1 << 20)  # a few alignments per pass
        got = a.align_many(refs, alts, SWG.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS)
        st = a.last_stats()
        assert st["chunks"] > 10
    _assert_same(got, refs, alts, S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS, S.SOFTCLIP, True)


def test_stats_count_shortcuts_and_cells(aligner):
    refs = [b"ACGTACGTAC", b"ACGTACGTAC", b"TTTTGGGG"]
    alts = [b"GTAC", b"GTTC", b"CCCC"]
    aligner.align_many(refs, alts, SWG.ORIGINAL_DEFAULT)
    st = aligner.last_stats()
    assert st["n_alignments"] == 3 and st["n_shortcut"] == 1
    assert st["cells"] == 10 * 4 + 8 * 4


def test_errors_are_the_references(aligner):
    with pytest.raises(ValueError, match="non-empty sequences"):
        aligner.align_native(b"", b"ACGT", SWG.ORIGINAL_DEFAULT, SWG.SWOverhangStrategy.SOFTCLIP)
    with pytest.raises(ValueError, match="non-empty sequences"):
        aligner.align_many([b"ACGT", b"AC"], [b"A", b""], SWG.ORIGINAL_DEFAULT)
    with pytest.raises(ValueError, match="overhang strategy"):
        aligner.align_native(b"ACGT", b"AC", SWG.ORIGINAL_DEFAULT, 7)
    # the context keeps working after an error
    a = aligner.align(b"AAACCCCC", b"CCCCC", SWG.ORIGINAL_DEFAULT, SWG.SWOverhangStrategy.INDEL)
    assert (a.cigar, a.alignment_offset) == ("3D5M", 0)


def test_cigar_capacity_is_checked(aligner):
    pairs = (native.SwPair * 1)()
    r, a = np.frombuffer(b"ACGTTT", np.uint8), np.frombuffer(b"AGT", np.uint8)
    pairs[0] = native.SwPair(r.ctypes.data, a.ctypes.data, 6, 3)
    res, off, start, length, ops = SWG._result(1, 0)
    p = SWG.ORIGINAL_DEFAULT.as_native()
    rc = aligner._ctx.L.ghmm_sw_align_batch(aligner.handle, pairs, 1, p, 0, 0, res)
    assert rc == native.GHMM_ERR_ARG
    assert "cigar_cap" in native.last_error(aligner.handle)


def _realign_oracle(wl, out, prio, params):
    refs, alts, best, inf = [], [], [], []
    for g in range(wl.n_regions):
        h0, h1 = int(wl.region_hap_off[g]), int(wl.region_hap_off[g + 1])
        nh = h1 - h0
        o = int(wl.out_off[g])
        for k, r in enumerate(range(int(wl.region_read_off[g]), int(wl.region_read_off[g + 1]))):
            row = out[o + k * nh:o + (k + 1) * nh]
            b, i = P.best_allele_breaking_ties(list(row), None if prio is None else list(prio[h0:h1]))
            best.append(b)
            inf.append(i)
            h = h0 + b
            refs.append(bytes(wl.hap_bases[int(wl.hap_off[h]):int(wl.hap_off[h + 1])]))
            alts.append(bytes(wl.bases[int(wl.read_off[r]):int(wl.read_off[r + 1])]))
    return refs, alts, np.array(best), np.array(inf)


@pytest.mark.parametrize("with_priority", [False, True])
def test_realign_reads_to_their_best_haplotype(engine, with_priority):
    from gatk_gb300.pairhmm import Batch

    wl = W.generate(1, regions=12, seed=41)
    prio = None
    if with_priority:
        rng = np.random.default_rng(3)
        prio = rng.integers(-3, 2, size=wl.n_haps).astype(np.float64)
    with Batch(engine, wl) as b:
        b.forward()
        out = b.results()
        best, inf, got = SWG.realign_batch(b, prio)
    refs, alts, exp_best, exp_inf = _realign_oracle(wl, out, prio, S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS)
    np.testing.assert_array_equal(best, exp_best)
    np.testing.assert_array_equal(inf, exp_inf)
    _assert_same(got, refs, alts, S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS, S.SOFTCLIP, True)


def test_realign_after_postprocess_uses_the_normalised_likelihoods(engine):
    from gatk_gb300.pairhmm import Batch

    wl = W.generate(1, regions=6, seed=43)
    with Batch(engine, wl) as b:
        b.forward()
        b.postprocess(cap=-0.5, symmetric=True)
        out = b.results()
        best, inf, got = SWG.realign_batch(b, np.zeros(wl.n_haps))
    refs, alts, exp_best, exp_inf = _realign_oracle(wl, out, np.zeros(wl.n_haps),
                                                     S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS)
    np.testing.assert_array_equal(best, exp_best)
    np.testing.assert_array_equal(inf, exp_inf)
    _assert_same(got, refs, alts, S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS, S.SOFTCLIP, True)


def test_int16_pairs_and_int32_give_the_oracle_alignments():
    # bounded alignments run two per warp in 16-bit halves by default; the int32-only option runs the same ones
    # one per warp; both must equal the oracle (an odd number per width leaves a half empty)
    rng = random.Random(31)
    refs, alts = _pairs(rng, 501, (40, 620), (1, 256))
    params = S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS
    with SWG.SmithWatermanCudaAligner() as a:
        for st in (S.SOFTCLIP, S.INDEL):
            a.set_int32_only(False)
            got16 = a.align_many(refs, alts, SWG.SWParameters(*params), SWG.SWOverhangStrategy(st))
            s16 = a.last_stats()
            a.set_int32_only(True)
            got32 = a.align_many(refs, alts, SWG.SWParameters(*params), SWG.SWOverhangStrategy(st))
            s32 = a.last_stats()
            assert s16["n_int16"] > 300 and s32["n_int16"] == 0
            _assert_same(got16, refs, alts, params, st, True)
            _assert_same(got32, refs, alts, params, st, True)


def test_unbounded_scores_stay_in_int32(aligner):
    # NEW_SW_PARAMETERS' match value of 200 over a 256-column alt could leave the 16-bit range: int32 kernel
    rng = random.Random(32)
    refs, alts = _pairs(rng, 60, (300, 500), (200, 256))
    got = aligner.align_many(refs, alts, SWG.NEW_SW_PARAMETERS, SWG.SWOverhangStrategy.SOFTCLIP, False)
    assert aligner.last_stats()["n_int16"] == 0
    _assert_same(got, refs, alts, S.NEW_SW_PARAMETERS, S.SOFTCLIP, False)


def _native_pairs(ref_buf, ref_pos, ref_len, alts):
    """SwPair array of refs at ref_buf[ref_pos[i]:ref_pos[i] + ref_len[i]] against alts (kept alive by the caller)."""
    abuf = np.frombuffer(b"".join(alts), dtype=np.uint8)
    aoff = np.cumsum([0] + [len(a) for a in alts])
    pairs = (native.SwPair * len(alts))()
    for i in range(len(alts)):
        pairs[i] = native.SwPair(ref_buf.ctypes.data + int(ref_pos[i]), abuf.ctypes.data + int(aoff[i]),
                                 int(ref_len[i]), len(alts[i]))
    return pairs, abuf


def test_batch_call_shares_refs_across_blocks_of_pairs(aligner):
    # 20,000 pairs: the call checks and deduplicates its refs in several blocks of pairs at once.  Six haplotypes in
    # one buffer, every block pointing at the same ones, three pairs in ten at a prefix of one (the same address with a
    # shorter length, a different ref); the alignments must equal the oracle's on the same bytes
    rng = random.Random(41)
    haps = [bytes(rng.choice(b"ACGT") for _ in range(rng.randint(150, 300))) for _ in range(6)]
    buf = np.frombuffer(b"".join(haps), dtype=np.uint8)
    hoff = np.cumsum([0] + [len(h) for h in haps])
    refs, alts, pos, lens = [], [], [], []
    for _ in range(20000):
        h = rng.randrange(len(haps))
        n_ref = len(haps[h]) if rng.random() < 0.7 else rng.choice((60, 100, 140))
        ref = haps[h][:n_ref]
        m = rng.randint(20, min(120, n_ref))
        a0 = rng.randint(0, n_ref - m)
        alt = _mutate(rng, ref[a0:a0 + m], b"ACGT", 0.03, 0.01) or b"A"
        refs.append(ref)
        alts.append(alt)
        pos.append(hoff[h])
        lens.append(n_ref)
    pairs, keep = _native_pairs(buf, pos, lens, alts)
    n = len(alts)
    L = aligner._ctx.L
    res, off, start, length, ops = SWG._result(n, int(L.ghmm_sw_cigar_bound(pairs, n)))
    p = S.ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS
    native.check(L.ghmm_sw_align_batch(aligner.handle, pairs, n, SWG.SWParameters(*p).as_native(), S.SOFTCLIP,
                                       native.SW_SUBSTRING_SHORTCUT, res), aligner.handle)
    got = SWG.AlignmentBatch(off[:n], start[:n], length[:n], ops[:res.cigar_total])
    _assert_same(got, refs, alts, p, S.SOFTCLIP, True)
    # each of the 24 distinct refs goes up once per block, not once per pair (besides the planes: 64-byte pairs up
    # twice and once more per pass, at most 8 task bytes a pair)
    assert aligner.last_stats()["h2d_bytes"] < sum(len(a) for a in alts) + sum(lens) // 4 + 200 * n


def test_batch_call_reports_the_first_bad_pair(aligner):
    # a ref longer than GHMM_SW_MAX_LEN at pair 9,000 and an empty alt at pair 15,000, in different blocks of the
    # call's parallel checks: the first one is reported, and nothing is aligned
    n, max_len = 20000, 1 << 20
    buf = np.frombuffer(b"ACGT" * (max_len // 4 + 1), dtype=np.uint8)
    lens = [40] * n
    lens[9000] = max_len + 1
    alts = [b"CGTACGTA"] * n
    pairs, keep = _native_pairs(buf, [0] * n, lens, alts)
    pairs[15000] = native.SwPair(buf.ctypes.data, None, 40, 0)
    L = aligner._ctx.L
    res, off, start, length, ops = SWG._result(n, int(4 * n * 16))
    p = SWG.ORIGINAL_DEFAULT.as_native()
    rc = L.ghmm_sw_align_batch(aligner.handle, pairs, n, p, S.SOFTCLIP, 0, res)
    assert rc == native.GHMM_ERR_ARG and "GHMM_SW_MAX_LEN" in native.last_error(aligner.handle)
    pairs[9000] = native.SwPair(buf.ctypes.data, keep.ctypes.data, 40, 8)
    rc = L.ghmm_sw_align_batch(aligner.handle, pairs, n, p, S.SOFTCLIP, 0, res)
    assert rc == native.GHMM_ERR_ARG and "non-empty sequences" in native.last_error(aligner.handle)
    pairs[15000] = native.SwPair(buf.ctypes.data, keep.ctypes.data, 40, 8)
    native.check(L.ghmm_sw_align_batch(aligner.handle, pairs, n, p, S.SOFTCLIP, 0, res), aligner.handle)
    assert len(set(off[:n].tolist())) == 1 and len(set(length[:n].tolist())) == 1
