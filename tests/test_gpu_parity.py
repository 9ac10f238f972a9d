"""GPU parity of the CUDA path against the FP64 oracle, through the C-ABI (libghmm.so).

Tolerances (|delta log10 L| against LoglessPairHMM in FP64 on the same inputs):
  FP32 batched path        <= 1e-3 (budget); on the reference's vector test data <= 1e-5, the bar the
                           reference sets for its native FP32 implementation (VectorPairHMMUnitTest.java:100)
  FP64 path (reruns/mode)  <= 1e-9
  plain FP64 kernel        <= 1e-12 (Java's operation order; only the final log10 may differ in the last ulp)
"""
import math

import numpy as np
import pytest

from conftest import load_golden
from gatk_gb300 import native, workload as W
from gatk_gb300.pairhmm import CudaLoglessPairHMM, Engine, PairHMMNativeArguments
from oracle import oracle as O

pytestmark = pytest.mark.gpu

TOL32 = 1e-3
TOL64 = 1e-9
TOL_PLAIN = 1e-12
# log10 L below which the FP32 scaled sum (L * 2^120) is under the 1e-28 rerun threshold
RERUN_LOG10 = math.log10(1e-28) - 120 * math.log10(2)


def _golden_workload(name):
    rows = load_golden(name)
    regions = [([h], [(r, q, i, d, g)]) for h, r, q, i, d, g, _ in rows]
    return W.from_pairs(regions), np.array([float(r[6]) for r in rows]), rows


def _oracle_all(wl):
    return O.compute_workload(wl)


def _absdiff(got, ref):
    """|got - ref| where equal infinities count as 0 (a pair whose likelihood underflows even the FP64
    2^1020 scale is -Infinity in LoglessPairHMM too); any other non-finite value is an error."""
    got = np.asarray(got)
    ref = np.asarray(ref)
    same_inf = np.isinf(got) & np.isinf(ref) & (got == ref)
    with np.errstate(invalid="ignore"):
        d = np.where(same_inf, 0.0, np.abs(got - ref))
    assert not np.isnan(d).any(), "non-finite result where the oracle has a finite one"
    return d


def _run(engine, wl, mode):
    with engine.batch(wl) as b:
        b.forward(mode)
        return b.results(), b.stats()


@pytest.mark.parametrize("name", ["hc_java_hmmresults.tsv", "vector_pairhmm_testdata.tsv"])
def test_golden_fp32(engine, name):
    wl, expected, _ = _golden_workload(name)
    got, st = _run(engine, wl, native.MODE_FP32_RERUN)
    ref = _oracle_all(wl)
    assert np.max(_absdiff(got, ref)) <= 1e-5
    assert np.max(_absdiff(got, expected)) <= 1e-5
    assert st["n_rerun"] == 0


@pytest.mark.parametrize("name", ["hc_java_hmmresults.tsv", "vector_pairhmm_testdata.tsv"])
def test_golden_fp64_and_plain(engine, name):
    wl, expected, rows = _golden_workload(name)
    ref = _oracle_all(wl)
    got64, _ = _run(engine, wl, native.MODE_FP64)
    assert np.max(_absdiff(got64, ref)) <= TOL64
    plain, _ = _run(engine, wl, native.MODE_PLAIN_FP64)
    assert np.max(_absdiff(plain, ref)) <= TOL_PLAIN
    if name.startswith("hc_java"):
        # the reference's own LOGLESS_CACHING dump matches as printed text
        assert all("%e" % v == r[6] for v, r in zip(plain, rows))


def test_workload0_all_modes(engine):
    wl = W.generate(0)
    ref = _oracle_all(wl)
    got32, st = _run(engine, wl, native.MODE_FP32_RERUN)
    d = _absdiff(got32, ref)
    assert d.max() <= TOL32 and np.median(d) <= 1e-5
    assert st["n_cells"] == wl.cells()
    got64, _ = _run(engine, wl, native.MODE_FP64)
    assert _absdiff(got64, ref).max() <= TOL64
    plain, _ = _run(engine, wl, native.MODE_PLAIN_FP64)
    assert _absdiff(plain, ref).max() <= TOL_PLAIN


def test_workload1_subsample(engine):
    wl = W.generate(1, regions=24)
    ref = _oracle_all(wl)
    got, st = _run(engine, wl, native.MODE_FP32_RERUN)
    d = _absdiff(got, ref)
    assert d.max() <= TOL32, d.max()
    assert np.median(d) <= 1e-5
    rerun = st["n_rerun"]
    if rerun:
        # pairs the FP32 pass handed to FP64 (scaled sum < 1e-28, i.e. log10 L < -64.12) are FP64-exact
        small = ref < RERUN_LOG10 - 0.01
        assert _absdiff(got[small], ref[small]).max() <= TOL64


def test_workload2_rerun_path(engine):
    wl = W.generate(2, regions=2)
    ref = _oracle_all(wl)
    # with the predicted-underflow routing off, every underflowing pair goes through the FP32 pass and its rerun
    engine.set_tuning(route_fp64_below=-1000000)
    try:
        got, st = _run(engine, wl, native.MODE_FP32_RERUN)
    finally:
        engine.set_tuning(route_fp64_below=0)  # back to the default
    assert st["n_rerun"] > 0 and st["n_fp64_direct"] == 0
    d = _absdiff(got, ref)
    # reruns are the underflowing pairs (log10 L below about -64)
    under = ref < RERUN_LOG10 - 0.01
    assert _absdiff(got[under], ref[under]).max() <= TOL64
    assert d.max() <= TOL32
    # with the routing on (the default), reads expected far below the FP32 range skip the FP32 pass.  A pair's FP64
    # result does not depend on the way it reached the FP64 kernel, so every rerun pair keeps its bits; the pairs
    # that change are FP32 results now computed in FP64
    got2, st2 = _run(engine, wl, native.MODE_FP32_RERUN)
    assert st2["n_fp64_direct"] > 0 and st2["n_cells_fp64_direct"] > 0
    assert st2["n_rerun"] + st2["n_fp64_direct"] >= st["n_rerun"]
    assert np.array_equal(got2[under], got[under])
    changed = got2 != got
    assert _absdiff(got2[changed], ref[changed]).max(initial=0.0) <= TOL64
    assert _absdiff(got2, ref).max() <= TOL32


def test_predicted_underflow_routing_leaves_workload1_alone(engine):
    wl = W.generate(1, regions=60)
    got, st = _run(engine, wl, native.MODE_FP32_RERUN)
    assert st["n_fp64_direct"] == 0  # reads of 100-250 bases at Q10-40 are far above the routing bound
    assert _absdiff(got, _oracle_all(wl)).max() <= TOL32


def _single(hap, read, q=30, ins=45, dl=45, gcp=10):
    n = len(read)
    arr = lambda v: np.full(n, v, dtype=np.uint8) if np.isscalar(v) else np.asarray(v, dtype=np.uint8)
    return ([hap], [(read, arr(q), arr(ins), arr(dl), arr(gcp))])


def _rand_seq(rng, n):
    return bytes(rng.choice(list(b"ACGT"), size=n).astype(np.uint8))


def test_strip_and_bucket_boundaries(engine):
    # read lengths around every rows-per-lane bucket edge (32k) and the multi-strip switch (256)
    rng = np.random.default_rng(7)
    regions = []
    for R in [1, 2, 3, 31, 32, 33, 63, 64, 65, 95, 96, 97, 127, 128, 129, 160, 191, 192, 193, 224, 225, 255, 256,
              257, 300, 511, 512, 513, 700]:
        hap = _rand_seq(rng, R + 40)
        read = bytearray(hap[20:20 + R])
        for k in rng.integers(0, R, size=max(1, R // 50)):
            read[k] = ord("ACGT"[(b"ACGT".index(read[k]) + 1) % 4])
        q = rng.integers(20, 41, size=R)
        regions.append(([hap, _rand_seq(rng, R + 5)], [(bytes(read), q, np.full(R, 45), np.full(R, 45), np.full(R, 10)),
                                                      (bytes(read[::-1]), q, np.full(R, 40), np.full(R, 43), np.full(R, 10))]))
    wl = W.from_pairs(regions)
    ref = _oracle_all(wl)
    got, _ = _run(engine, wl, native.MODE_FP32_RERUN)
    under = ref < RERUN_LOG10 - 0.01
    assert _absdiff(got[~under], ref[~under]).max() <= TOL32
    assert _absdiff(got[under], ref[under]).max() <= TOL64


@pytest.mark.parametrize("tuning", [(8, 8), (6, 4), (4, 2), (2, 1), (5, 3)])
def test_tunings_agree_with_oracle(tuning):
    # every launch shape (rows per lane, strips) gives the same results; reads of one region cover
    # several strip counts so pairs of reads with different strip counts would be exposed
    rng = np.random.default_rng(29)
    regions = []
    for _ in range(3):
        H = int(rng.integers(150, 400))
        base = _rand_seq(rng, H)
        haps = [base, base[:H // 2] + b"T" + base[H // 2 + 1:], _rand_seq(rng, H - 7)]
        reads = []
        for R in (100, 130, 161, 190, 200, 229, 250, 257, 300):
            start = int(rng.integers(0, max(1, H - R)))
            rd = (base[start:start + R] + _rand_seq(rng, R))[:R]
            reads.append((rd, rng.integers(20, 41, size=R), np.full(R, 45), np.full(R, 45), np.full(R, 10)))
        regions.append((haps, reads))
    wl = W.from_pairs(regions)
    ref = _oracle_all(wl)
    e = Engine()
    try:
        e.set_tuning(*tuning)
        got, _ = _run(e, wl, native.MODE_FP32_RERUN)
    finally:
        e.close()
    under = ref < RERUN_LOG10 - 0.01
    assert _absdiff(got[~under], ref[~under]).max() <= TOL32
    if under.any():
        assert _absdiff(got[under], ref[under]).max() <= TOL64


def test_results_do_not_depend_on_launch_shape():
    # a read's FP32 result is the same bits whatever rows per lane, strips, haplotype chunks or task partner it gets
    # (its row rescaling log2 a_R is summed by the read alone, dummy rows above it reproduce the row-0 boundary)
    wl = W.generate(1, regions=30)
    outs = []
    for tuning in ((8, 8, 16384), (4, 2, 1000), (6, 3, 300), (2, 1, 64)):
        e = Engine()
        try:
            e.set_tuning(*tuning)
            outs.append(_run(e, wl, native.MODE_FP32_RERUN)[0])
        finally:
            e.close()
    for o in outs[1:]:
        assert np.array_equal(o, outs[0])
    assert _absdiff(outs[0], _oracle_all(wl)).max() <= TOL32


def test_reads_longer_than_haplotypes_across_haplotype_boundaries(engine):
    # Every haplotype but the last hands the wavefront to the next one mid-warp; reads longer than the
    # haplotypes make the insertion chain at each haplotype's last column dominate the likelihood.
    rng = np.random.default_rng(19)
    regions = []
    for R, H in ((240, 225), (247, 219), (60, 40), (33, 31), (150, 100), (300, 280)):
        base = _rand_seq(rng, H)
        haps = [base, base[:H - 3] + b"ACG", _rand_seq(rng, H - 5)]
        reads = []
        for _ in range(3):
            rd = bytearray(base + _rand_seq(rng, R - H))
            q = rng.integers(10, 41, size=R)
            reads.append((bytes(rd), q, np.full(R, 45), np.full(R, 45), np.full(R, 10)))
        regions.append((haps, reads))
    wl = W.from_pairs(regions)
    ref = _oracle_all(wl)
    got, _ = _run(engine, wl, native.MODE_FP32_RERUN)
    under = ref < RERUN_LOG10 - 0.01
    assert _absdiff(got[~under], ref[~under]).max() <= TOL32
    if under.any():
        assert _absdiff(got[under], ref[under]).max() <= TOL64


def test_odd_reads_short_haps_and_long_reads(engine):
    rng = np.random.default_rng(11)
    regions = []
    for nr in (1, 3, 5):
        haps = [_rand_seq(rng, int(h)) for h in rng.integers(1, 60, size=3)]
        reads = []
        for _ in range(nr):
            R = int(rng.integers(1, 90))
            reads.append((_rand_seq(rng, R), rng.integers(10, 41, size=R), np.full(R, 45), np.full(R, 45), np.full(R, 10)))
        regions.append((haps, reads))
    wl = W.from_pairs(regions)
    ref = _oracle_all(wl)
    got, _ = _run(engine, wl, native.MODE_FP32_RERUN)
    under = ref < RERUN_LOG10 - 0.01
    assert _absdiff(got[~under], ref[~under]).max() <= TOL32
    if under.any():
        assert _absdiff(got[under], ref[under]).max() <= TOL64


def test_known_answer_cases_with_anchored_penalties(engine):
    # PairHMMUnitTest.java:148-199 cases: penalties of 100 everywhere except at the indel, so insertion
    # penalties rise steeply between neighbouring positions (the FP32 kernel's rescaled insertion state is
    # bounded on the host and such reads go to FP64 when the bound could exceed FP32's range)
    ctx = b"ACGTAATGACGATTGCA"
    regions = []
    for bq, iq, gcp in ((10, 20, 8), (30, 40, 10), (50, 50, 20)):
        for size in (2, 5, 10, 35):
            for ins in (True, False):
                small, big = b"A", b"A" * size
                ref, read = (small, big) if ins else (big, small)
                hap = ctx + ref + ctx
                rd = ctx + read + ctx
                n = len(rd)
                q = np.full(n, 100, dtype=np.uint8)
                q[len(ctx):len(ctx) + len(read)] = bq
                g = np.full(n, 100, dtype=np.uint8)
                g[len(ctx)] = iq
                c = np.full(n, 100, dtype=np.uint8)
                c[len(ctx):len(ctx) + len(read)] = gcp
                regions.append(([hap], [(rd, q, g, g, c)]))
    wl = W.from_pairs(regions)
    ref = _oracle_all(wl)
    got, st = _run(engine, wl, native.MODE_FP32_RERUN)
    assert np.isfinite(got).all()
    assert _absdiff(got, ref).max() <= TOL32


def test_special_bytes_route_to_fp64(engine):
    # N bases, gap continuation 0 and non-ACGTN bytes: results are exact FP64
    rng = np.random.default_rng(3)
    hap = _rand_seq(rng, 80)
    read = bytearray(hap[10:60])
    read[5] = ord("N")
    read_r = bytearray(read)
    read_r[7] = ord("R")
    gcp0 = np.full(50, 10)
    gcp0[20] = 0
    hapn = bytearray(hap)
    hapn[30] = ord("N")
    regions = [
        _single(hap, bytes(read)),
        _single(bytes(hapn), bytes(read)),
        _single(hap, bytes(read_r)),
        _single(hap, bytes(read), gcp=gcp0),
        _single(b"ACGTRACGT" + hap[:40], bytes(read)),
    ]
    wl = W.from_pairs(regions)
    ref = _oracle_all(wl)
    got, st = _run(engine, wl, native.MODE_FP32_RERUN)
    assert st["n_fp64_direct"] == 3
    assert _absdiff(got[2:], ref[2:]).max() <= TOL64
    assert _absdiff(got[:2], ref[:2]).max() <= TOL32


def test_empty_read_and_haplotype(engine):
    wl = W.from_pairs([
        ([b"ACGTACGT"], [(b"", [], [], [], [])]),
        ([b""], [(b"ACG", [30, 30, 30], [45] * 3, [45] * 3, [10] * 3)]),
    ])
    got, _ = _run(engine, wl, native.MODE_FP32_RERUN)
    assert np.all(got == -np.inf)


def test_quality_out_of_range_is_an_argument_error(engine):
    for q, ins in ((255, 45), (30, 128)):
        wl = W.from_pairs([_single(b"ACGTACGT", b"ACGT", q=q, ins=ins)])
        with pytest.raises(native.GhmmError) as e:
            engine.compute(wl)
        assert e.value.code == native.GHMM_ERR_ARG


def test_entry_points_agree(engine):
    wl = W.generate(1, regions=6)
    a = engine.compute(wl)
    b = engine.compute(wl, via_regions=True)
    with engine.batch(wl, via_regions=True) as bt:
        bt.forward()
        c = bt.results()
    assert np.array_equal(a, b) and np.array_equal(a, c)


def test_repeated_forward_is_deterministic(engine):
    wl = W.generate(1, regions=8)
    with engine.batch(wl) as b:
        b.forward()
        x = b.results()
        b.forward()
        y = b.results()
    assert np.array_equal(x, y)


def test_pairhmm_interface_known_answer():
    # PairHMMUnitTest.testLikelihoodsFromHaplotypes (PairHMMUnitTest.java:512-537): 10 A's vs 20 A's
    hmm = CudaLoglessPairHMM(PairHMMNativeArguments())
    try:
        hmm.initialize([b"A" * 20])
        assert hmm.compute_log10_likelihoods([]) is None
        la = hmm.compute_log10_likelihoods([(b"A" * 10, [20] * 10, [45] * 10, [45] * 10, [100] * 10)])
        assert la.shape == (1,)
        expected = math.log10((20 - 10 + 1) / 20 * (1 - 10 ** -2.0) ** 10)
        assert abs(la[0] - expected) <= 1e-3
    finally:
        hmm.close()


def test_pairhmm_interface_read_major_matrix():
    wl = W.generate(0)
    haps = [wl.hap(h) for h in range(wl.n_haps)]
    reads = [wl.read(r) for r in range(wl.n_reads)]
    with CudaLoglessPairHMM() as hmm:
        hmm.initialize(haps)
        la = hmm.compute_log10_likelihoods(reads)
    ref = _oracle_all(wl)
    assert la.shape == ref.shape
    assert _absdiff(la, ref).max() <= TOL32


def test_double_precision_argument():
    wl = W.generate(0)
    e = Engine(use_double_precision=True)
    try:
        got = e.compute(wl)
    finally:
        e.close()
    assert _absdiff(got, _oracle_all(wl)).max() <= TOL64


def test_peaks_are_sane(engine):
    p = engine.measure_peaks()
    assert 20 < p["fp32_tflops"] < 200
    assert 20 < p["fp32x2_tflops"] < 400
    assert 0 < p["fp64_tflops"] < 100


def test_fp64_tiers_near_the_bottom_of_the_range(engine):
    # random reads against unrelated haplotypes at low base quality: log10 L from about -150 to below the
    # FP64 range (-Infinity in LoglessPairHMM too); results below the rescaled tier's floor (-560) come
    # from the exact tier, and everything matches the oracle to the FP64 bar
    rng = np.random.default_rng(11)
    regions = []
    for R in (150, 250, 350, 450, 550, 650, 800, 1200):
        hap = _rand_seq(rng, R + 40)
        regions.append(_single(hap, _rand_seq(rng, R), q=rng.integers(8, 14, size=R)))
    wl = W.from_pairs(regions)
    ref = _oracle_all(wl)
    assert (ref < native.FP64_RESCALED_FLOOR).any() and (ref > native.FP64_RESCALED_FLOOR).any()
    for mode in (native.MODE_FP32_RERUN, native.MODE_FP64):
        got, st = _run(engine, wl, mode)
        finite = np.isfinite(ref) & (ref > -600)
        assert np.abs(got[finite] - ref[finite]).max() <= TOL64, mode
        # at the very bottom (subnormal sums) the reference itself is imprecise; only the -Infinity
        # boundary is compared there
        deep = ~finite
        assert np.all((got[deep] == -np.inf) | (got[deep] < -600)), mode
        assert st["n_fp64_exact"] >= int((ref < native.FP64_RESCALED_FLOOR).sum()), mode


def test_insertion_growth_routes_to_the_exact_tier(engine):
    # the rescaled forms carry 1 / MI, so a read's insertion state can grow by err(gcp) err(ins_prev) / (err(ins) MM_prev)
    # per row.  A read whose bound on that growth passes 1e15 (low, flat gap penalties: about 7e30 here) goes to the
    # exact FP64 tier; one whose bound stays under it (an insertion penalty jumping 10 -> 127 at every other base: about
    # 6e10) runs in the rescaled FP64 tier, inside its 2^60 headroom.  Both match the oracle to the FP64 bar.
    rng = np.random.default_rng(5)
    hap = _rand_seq(rng, 120)
    read = hap[20:90]
    ins = np.where(np.arange(70) % 2 == 0, 10, 127)
    wl = W.from_pairs([_single(hap, read, ins=ins), _single(hap, read, ins=4, dl=5, gcp=1), _single(hap, read)])
    ref = _oracle_all(wl)
    got, st = _run(engine, wl, native.MODE_FP32_RERUN)
    assert st["n_fp64_exact"] == 1 and st["n_fp64_direct"] == 2
    assert _absdiff(got[:2], ref[:2]).max() <= TOL64
    assert _absdiff(got[2:], ref[2:]).max() <= TOL32


@pytest.mark.gpu
def test_exhaustive_small_shapes(engine):
    # every read length on a grid around the 32-row lane and strip granularities against every haplotype length on
    # a grid around the 32-column wavefront width, one region per haplotype length, in FP32 and in FP64
    rng = np.random.default_rng(77)
    read_lens = (1, 2, 3, 5, 8, 13, 21, 29, 30, 31, 32, 33, 34, 62, 63, 64, 65, 66, 94, 126, 254, 255, 256)
    hap_lens = (1, 2, 3, 5, 8, 31, 32, 33, 63, 64, 65, 100)
    regions = []
    for H in hap_lens:
        haps = [_rand_seq(rng, H), _rand_seq(rng, H + 1)]
        reads = [(_rand_seq(rng, R), rng.integers(10, 41, size=R), rng.integers(20, 46, size=R),
                  rng.integers(20, 46, size=R), np.full(R, 10)) for R in read_lens]
        regions.append((haps, reads))
    wl = W.from_pairs(regions)
    ref = _oracle_all(wl)
    got, _ = _run(engine, wl, native.MODE_FP32_RERUN)
    under = ref < RERUN_LOG10 - 0.01
    assert _absdiff(got[~under], ref[~under]).max() <= TOL32
    if under.any():
        assert _absdiff(got[under], ref[under]).max() <= TOL64
    got64, _ = _run(engine, wl, native.MODE_FP64)
    assert _absdiff(got64, ref).max() <= TOL64
