"""Read preparation before the PairHMM (PairHMMLikelihoodCalculationEngine.modifyReadQualities, the PCR indel
error model with findTandemRepeatUnits, standard imputation, DRAGstr imputation): the CPU restatement
oracle/readprep.py against the reference's own unit-test cases, and the device path (ghmm_compute_regions_raw)
against the regular forward on the restatement's prepared planes (identical planes give identical results)."""
import json
import os

import numpy as np
import pytest

from gatk_gb300 import workload as W
from oracle import readprep as RP


def test_repetitions_match_the_reference_cases():
    # GATKVariantContextUtilsUnitTest.java:923-927
    assert RP.repetitions(b"AT", b"GATAT", False) == 2
    assert RP.repetitions(b"AT", b"GATAT", True) == 0
    assert RP.repetitions(b"A", b"ATATG", True) == 1
    assert RP.repetitions(b"AT", b"ATATG", True) == 2
    assert RP.repetitions(b"CCC", b"CCCCCCCC", True) == 2


def test_tandem_repeat_lengths():
    assert RP.tandem_repeat_length(b"AAAA", 1) == 4          # inside a homopolymer run
    assert RP.tandem_repeat_length(b"ACACACGT", 1) == 3       # (AC)3 around the boundary at offset 1
    assert RP.tandem_repeat_length(b"A" * 30, 10) == 20       # capped at MAX_REPEAT_LENGTH
    assert RP.tandem_repeat_length(b"ACGT", 3) <= 1           # end of read, no repeat


@pytest.mark.parametrize("repeat", ["A", "AC", "ACG", "ACGT"])
@pytest.mark.parametrize("n", [1, 2, 3, 5, 10, 15])
def test_pcr_model_applies_the_cache(repeat, n):
    # PairHMMLikelihoodCalculationEngineUnitTest.createPcrErrorModelTest: insertion / deletion qualities of 40
    # capped to getErrorModelAdjustedQual(repeat length, CONSERVATIVE = 3.0)
    read = (repeat * n).encode()
    L = len(read)
    _, _, ins, dels, _ = RP.prepare_read(read, [40] * L, [40] * L, [40] * L, mapq=255, threshold=0, cap_to_mapq=False,
                                          rate_factor=3.0)
    cache = RP.pcr_cache(3.0)
    for i in range(1, L):
        want = cache[RP.tandem_repeat_length(read, i - 1)]
        assert ins[i - 1] == min(40, want) and dels[i - 1] == min(40, want)


def test_quality_caps():
    b, q, i, d, g = RP.prepare_read(b"ACGTA", [40, 10, 30, 200, 17], [3, 45, 7, 200, 6], None, mapq=25, threshold=18,
                                    cap_to_mapq=True, rate_factor=0.0, gcp=10)
    assert list(q) == [25, 6, 25, 25, 6]          # min(q, MAPQ), then < 18 -> 6
    assert list(i) == [6, 45, 7, 6, 6]            # < 6 -> 6, and 200 is a negative Java byte -> 6
    assert list(d) == [45] * 5 and list(g) == [10] * 5
    _, q2, _, _, _ = RP.prepare_read(b"AC", [200, 30], None, None, mapq=255, threshold=18, cap_to_mapq=True)
    assert list(q2) == [6, 30]                    # 200 survives the MAPQ cap but is negative as a Java byte


def _prepared_workload(wl, mapq, with_indel, rate, threshold=18, cap=True, gcp=10, dragstr=None):
    planes = [np.empty_like(wl.bases) for _ in range(4)]
    for r in range(wl.n_reads):
        a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
        _, q, i, d, g = RP.prepare_read(wl.bases[a:b], wl.quals[a:b], wl.ins[a:b] if with_indel else None,
                                        wl.dels[a:b] if with_indel else None, int(mapq[r]), threshold, cap, rate, gcp,
                                        dragstr=dragstr)
        for k, v in enumerate((q, i, d, g)):
            planes[k][a:b] = np.frombuffer(v, dtype=np.uint8)
    return W.Workload(region_read_off=wl.region_read_off, region_hap_off=wl.region_hap_off, read_off=wl.read_off,
                      bases=wl.bases, quals=planes[0], ins=planes[1], dels=planes[2], gcp=planes[3],
                      hap_off=wl.hap_off, hap_bases=wl.hap_bases, out_off=wl.out_off)


def _raw_workload(seed=4):
    wl = W.generate(1, regions=6)
    rng = np.random.default_rng(seed)
    # raw qualities spanning the caps: low base qualities, low and high indel qualities, a range of MAPQs
    wl.quals[:] = rng.integers(2, 45, size=len(wl.quals)).astype(np.uint8)
    wl.ins[:] = rng.integers(0, 50, size=len(wl.ins)).astype(np.uint8)
    wl.dels[:] = rng.integers(0, 50, size=len(wl.dels)).astype(np.uint8)
    mapq = rng.integers(10, 70, size=wl.n_reads)
    return wl, mapq


@pytest.mark.gpu
@pytest.mark.parametrize("with_indel,rate,cap", [(True, 3.0, True), (False, 1.0, False), (True, 0.0, True)])
def test_device_preparation_gives_the_restatements_planes(engine, with_indel, rate, cap):
    wl, mapq = _raw_workload()
    want = _prepared_workload(wl, mapq, with_indel, rate, cap=cap)
    with engine.raw_batch(wl, mapq, with_indel_quals=with_indel, pcr_rate_factor=rate, cap_to_mapq=cap) as b:
        bases, q, i, d, g = b.read_planes()
    assert np.array_equal(bases, wl.bases)
    assert np.array_equal(q, want.quals)
    assert np.array_equal(i, want.ins)
    assert np.array_equal(d, want.dels)
    assert np.array_equal(g, want.gcp)


@pytest.mark.gpu
def test_raw_path_likelihoods_match_the_prepared_planes():
    # in double precision every pair runs in FP64, so the raw path and the regular path on the restatement's
    # planes agree to the FP64 bar (the host routes pairs between the two FP64 tiers from raw qualities)
    from gatk_gb300.pairhmm import Engine

    e = Engine(use_double_precision=True)
    try:
        wl, mapq = _raw_workload(7)
        raw = e.compute_raw(wl, mapq, pcr_rate_factor=3.0)
        ref = e.compute(_prepared_workload(wl, mapq, True, 3.0))
        assert np.abs(raw - ref).max() <= 1e-9
    finally:
        e.close()


# ---- DRAGstr imputation (DragstrPairHMMInputScoreImputator) ----
_GOLDEN = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "dragstr_cases.json")))
EXAMPLE = (np.array(_GOLDEN["example_params"]["gop"]), np.array(_GOLDEN["example_params"]["gcp"]))


def test_str_analysis_matches_the_reference_empirical_case():
    # DragstrReadSTRAnalyzerTest.testCasesData (:58-66): most repeated period and repeat count (hex, capped at 15
    # by the digits, 20 by the reference's own repeat cap) at each of the first 98 positions
    case = _GOLDEN["str_empirical"]
    periods, repeats = RP.str_analyze(case["read"].encode(), 8)
    n = len(case["periods"])
    assert periods[:n] == case["periods"]
    assert [min(20, r) for r in repeats[:n]] == case["repeats"]


def _str_read(rng, n, max_unit=10, max_reps=25):
    """Random bases with planted tandem repeats (units of 1..max_unit bases)."""
    b = bytearray(rng.choice(list(b"ACGT"), size=n).astype(np.uint8).tobytes())
    pos = 0
    while pos < n:
        pos += int(rng.integers(0, 40))
        ul, reps = int(rng.integers(1, max_unit + 1)), int(rng.integers(2, max_reps + 1))
        unit = rng.choice(list(b"ACGT"), size=ul).astype(np.uint8).tobytes()
        for _ in range(reps):
            if pos >= n:
                break
            m = min(ul, n - pos)
            b[pos:pos + m] = unit[:m]
            pos += ul
    return bytes(b)


def test_str_analysis_matches_the_library_analyzer():
    # the oracle's window definition against ghmm_str_analyze (the run-length form) on reads with planted repeats
    from gatk_gb300 import native

    rng = np.random.default_rng(17)
    for n in (1, 2, 7, 40, 151):
        for max_period in (1, 3, 8):
            seq = _str_read(rng, n)
            a = np.frombuffer(seq, dtype=np.uint8).copy()
            bp, br = np.zeros(n, dtype=np.int32), np.zeros(n, dtype=np.int32)
            allr = np.zeros(max_period * n, dtype=np.int32)
            p32 = lambda x: x.ctypes.data_as(native._i32p)
            assert native.lib().ghmm_str_analyze(a.ctypes.data_as(native._u8p), n, max_period, p32(bp), p32(br),
                                                 p32(allr)) == 0
            periods, repeats = RP.str_analyze(seq, max_period)
            assert list(bp) == periods and list(br) == repeats


def test_java_round():
    # Math.round(double): half up, also for negative halves
    assert [RP.java_round(x) for x in (2.5, 2.49, -0.5, -0.51, 21.75, 1.25, 3.33, 0.0)] == [3, 2, 0, -1, 22, 1, 3, 0]


def test_dragstr_imputation_rules():
    gop, gcp = EXAMPLE
    # one base: only the end-of-read values
    assert RP.dragstr_impute(b"A", gop, gcp) == (bytes([45]), bytes([10]))
    # a homopolymer of 30: period 1, repeats 30 clamp to the table's last column (20 repeats)
    g, c = RP.dragstr_impute(b"A" * 30, gop, gcp)
    assert g[:-1] == bytes([round(min(40.0, gop[0][19]) + 0.0)]) * 29 and g[-1] == 45
    assert c[:-1] == bytes([RP.java_round(gcp[0][19])]) * 29 and c[-1] == 10
    # GOP capped at 40 (47.5 at period 1, one repeat) and GCP rounded half up (3.33 -> 3 at period 3)
    g, c = RP.dragstr_impute(b"ACGTTGCA", gop, gcp)
    assert max(g[:-1]) <= 40
    g3, c3 = RP.dragstr_impute(b"ACGACGACGACG", gop, gcp)
    periods, repeats = RP.str_analyze(b"ACGACGACGACG", 8)
    assert periods[0] == 3 and c3[0] == 3
    # the analysis runs periods up to the table's own count (DragstrReadSTRAnalyzer.of(read, maximumPeriod())), so
    # only the repeat index clamps: (AC)6 with a 2 x 5 table reads column 5
    small = (gop[:2, :5] + np.arange(5), gcp[:2, :5] + np.arange(5))
    g, c = RP.dragstr_impute(b"ACACACACACAC", *small)
    assert RP.str_analyze(b"ACACACACACAC", 2)[0][0] == 2
    assert c[0] == RP.java_round(gcp[1][4] + 4) and g[0] == RP.java_round(min(40.0, gop[1][4] + 4))
    # with one period only, the same read is period 1 with one repeat
    g1, c1 = RP.dragstr_impute(b"ACACACACACAC", gop[:1], gcp[:1])
    assert c1[0] == RP.java_round(gcp[0][0])


def test_dragstr_prepare_read_keeps_the_base_quality_rules():
    gop, gcp = EXAMPLE
    b, q, i, d, g = RP.prepare_read(b"ACGTA", [40, 10, 30, 200, 17], [3, 45, 7, 200, 6], None, mapq=25,
                                    dragstr=(gop, gcp))
    assert list(q) == [25, 6, 25, 25, 6]
    assert i == d and i[-1] == 45 and g[-1] == 10      # the imputed planes, not the BI / BD tags


def _dragstr_workload(seed=5, regions=6, read_len=None):
    wl = W.generate(1, regions=regions)
    rng = np.random.default_rng(seed)
    for r in range(wl.n_reads):
        a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
        wl.bases[a:b] = np.frombuffer(_str_read(rng, b - a), dtype=np.uint8)
    wl.quals[:] = rng.integers(2, 45, size=len(wl.quals)).astype(np.uint8)
    mapq = rng.integers(10, 70, size=wl.n_reads)
    return wl, mapq


def _one_region(reads, haps, rng):
    read_off = np.concatenate([[0], np.cumsum([len(r) for r in reads])]).astype(np.int64)
    hap_off = np.concatenate([[0], np.cumsum([len(h) for h in haps])]).astype(np.int64)
    bases = np.frombuffer(b"".join(reads), dtype=np.uint8).copy()
    q = lambda lo, hi: rng.integers(lo, hi, size=len(bases)).astype(np.uint8)
    return W.Workload(region_read_off=np.array([0, len(reads)], dtype=np.int64),
                      region_hap_off=np.array([0, len(haps)], dtype=np.int64), read_off=read_off, bases=bases,
                      quals=q(10, 41), ins=q(20, 46), dels=q(20, 46), gcp=np.full(len(bases), 10, dtype=np.uint8),
                      hap_off=hap_off, hap_bases=np.frombuffer(b"".join(haps), dtype=np.uint8).copy(),
                      out_off=np.array([0, len(reads) * len(haps)], dtype=np.int64))


@pytest.mark.gpu
@pytest.mark.parametrize("tables", ["example", "small", "wide"])
def test_device_dragstr_gives_the_restatements_planes(engine, tables):
    gop, gcp = EXAMPLE
    if tables == "small":      # fewer periods and repeats than the reads show: lookups clamp
        gop, gcp = gop[:3, :4].copy(), gcp[:3, :4].copy()
    elif tables == "wide":     # more periods than the default 8, values that round both ways
        rng = np.random.default_rng(3)
        gop = rng.uniform(10.0, 50.0, size=(12, 30)).round(2)
        gcp = rng.uniform(0.5, 12.0, size=(12, 30)).round(2)
    wl, mapq = _dragstr_workload()
    want = _prepared_workload(wl, mapq, True, 3.0, dragstr=(gop, gcp))
    with engine.raw_batch(wl, mapq, dragstr=(gop, gcp)) as b:
        bases, q, i, d, g = b.read_planes()
    assert np.array_equal(bases, wl.bases)
    assert np.array_equal(q, want.quals)
    assert np.array_equal(i, want.ins)
    assert np.array_equal(d, want.dels)
    assert np.array_equal(g, want.gcp)


@pytest.mark.gpu
def test_device_dragstr_long_reads(engine):
    # reads of 1..2000 bases: several warps' worth of positions per read, one block per read's shared memory
    rng = np.random.default_rng(11)
    lens = [1, 2, 31, 32, 33, 64, 700, 1024, 1025, 2000]
    reads = [_str_read(rng, n) for n in lens] + [b"A" * 300, b"AC" * 200, b"ACGTTGCA" * 40 + b"T"]
    hap = _str_read(rng, 2100)
    wl = _one_region(reads, [hap], rng)
    mapq = np.full(wl.n_reads, 60)
    gop, gcp = EXAMPLE
    want = _prepared_workload(wl, mapq, True, 3.0, dragstr=(gop, gcp))
    with engine.raw_batch(wl, mapq, dragstr=(gop, gcp)) as b:
        _, q, i, d, g = b.read_planes()
    assert np.array_equal(i, want.ins) and np.array_equal(d, want.dels) and np.array_equal(g, want.gcp)
    assert np.array_equal(q, want.quals)


@pytest.mark.gpu
def test_device_pcr_model_long_and_repetitive_reads(engine):
    # reads up to 1,024 bases are searched in shared memory through runs of base-equality masks, longer ones base by
    # base in place; both against findTandemRepeatUnits as restated
    rng = np.random.default_rng(12)
    lens = [1, 2, 3, 9, 31, 32, 33, 64, 700, 1023, 1024, 1025, 2000]
    reads = [_str_read(rng, n) for n in lens] + [b"A" * 300, b"AC" * 200, b"ACGTTGCA" * 40 + b"T", b"AAC" * 90,
                                                 b"A" * 1100]
    wl = _one_region(reads, [_str_read(rng, 2100)], rng)
    mapq = np.full(wl.n_reads, 60)
    want = _prepared_workload(wl, mapq, True, 3.0)
    with engine.raw_batch(wl, mapq, pcr_rate_factor=3.0) as b:
        _, q, i, d, g = b.read_planes()
    assert np.array_equal(i, want.ins) and np.array_equal(d, want.dels)
    assert np.array_equal(q, want.quals) and np.array_equal(g, want.gcp)


@pytest.mark.gpu
def test_dragstr_likelihoods_match_the_prepared_planes():
    # FP64: the raw DRAGstr path against the regular forward on the restatement's planes
    from gatk_gb300.pairhmm import Engine

    e = Engine(use_double_precision=True)
    try:
        wl, mapq = _dragstr_workload(9)
        raw = e.compute_raw(wl, mapq, dragstr=EXAMPLE)
        ref = e.compute(_prepared_workload(wl, mapq, True, 3.0, dragstr=EXAMPLE))
        assert np.abs(raw - ref).max() <= 1e-9
    finally:
        e.close()


@pytest.mark.gpu
def test_dragstr_fp32_path_within_tolerance(engine):
    # the default FP32 forward with its FP64 rerun, on DRAGstr planes, against FP64 of the same planes
    from gatk_gb300.pairhmm import Engine

    wl, mapq = _dragstr_workload(13)
    got = engine.compute_raw(wl, mapq, dragstr=EXAMPLE)
    e64 = Engine(use_double_precision=True)
    try:
        ref = e64.compute(_prepared_workload(wl, mapq, True, 3.0, dragstr=EXAMPLE))
    finally:
        e64.close()
    assert np.all(np.isfinite(got))
    assert np.abs(got - ref).max() <= 1e-3  # CUDA_LOGLESS FP32 bar (absolute, log10 space)


@pytest.mark.gpu
def test_device_dragstr_very_long_read(engine):
    # a read whose shared-memory arrays exceed the default 48 KB a block (one warp per block, opt-in size)
    rng = np.random.default_rng(41)
    reads = [_str_read(rng, 12000, max_reps=8), _str_read(rng, 300)]
    wl = _one_region(reads, [_str_read(rng, 400)], rng)
    mapq = np.full(wl.n_reads, 60)
    want = _prepared_workload(wl, mapq, True, 3.0, dragstr=EXAMPLE)
    with engine.raw_batch(wl, mapq, dragstr=EXAMPLE) as b:
        _, q, i, d, g = b.read_planes()
    assert np.array_equal(i, want.ins) and np.array_equal(g, want.gcp) and np.array_equal(q, want.quals)


@pytest.mark.gpu
def test_dragstr_read_length_limit(engine):
    # the imputation holds a read in shared memory: 28000 bases at most, longer reads are refused
    rng = np.random.default_rng(2)
    wl = _one_region([_str_read(rng, 28001)], [_str_read(rng, 300)], rng)
    with pytest.raises(Exception, match="28000"):
        engine.compute_raw(wl, np.full(1, 60), dragstr=EXAMPLE)


@pytest.mark.gpu
@pytest.mark.parametrize("bad", ["nan", "negative_gcp", "gcp_too_large", "period_count"])
def test_dragstr_rejects_bad_tables(engine, bad):
    gop, gcp = EXAMPLE[0].copy(), EXAMPLE[1].copy()
    if bad == "nan":
        gop[2, 3] = np.nan
    elif bad == "negative_gcp":
        gcp[0, 0] = -3.0
    elif bad == "gcp_too_large":
        gcp[1, 1] = 128.0
    else:
        gop, gcp = np.ones((33, 4)) * 30, np.ones((33, 4)) * 10
    wl, mapq = _dragstr_workload()
    with pytest.raises(Exception, match="DRAGstr"):
        engine.compute_raw(wl, mapq, dragstr=(gop, gcp))


# ---- raw reads through the streaming queue (ghmm_queue_create_raw / ghmm_queue_push_raw) ----
@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["pcr", "dragstr"])
def test_raw_queue_matches_the_raw_call(engine, kind):
    # small batches, so that the regions spread over several batches and both buffer slots
    if kind == "pcr":
        wl, mapq = _raw_workload(21)
        kw = {"pcr_rate_factor": 3.0}
    else:
        wl, mapq = _dragstr_workload(22)
        kw = {"dragstr": EXAMPLE}
    want = engine.compute_raw(wl, mapq, **kw)
    q = engine.raw_queue(wl, batch_cells=int(wl.cells() // 3) + 1, **kw)
    try:
        got = q.push_raw(wl, mapq)
        q.flush()
        info = q.info()
    finally:
        q.close()
    assert info["n_batches"] >= 3 and info["n_regions"] == wl.n_regions
    assert np.array_equal(got, want)


@pytest.mark.gpu
def test_raw_and_plain_queues_take_their_own_pushes(engine):
    from gatk_gb300 import native

    wl, mapq = _raw_workload(23)
    rq = engine.raw_queue(wl)
    try:
        with pytest.raises(native.GhmmError, match="ghmm_queue_push_raw"):
            rq.push(wl)
        rq.push_raw(wl, mapq)  # the rejected push left the queue usable
        rq.flush()
    finally:
        rq.close()
    pq = engine.queue()
    try:
        with pytest.raises(native.GhmmError, match="ghmm_queue_create_raw"):
            pq.push_raw(wl, mapq)
    finally:
        pq.close()


@pytest.mark.gpu
def test_raw_queue_rejects_bad_reads_at_push(engine):
    from gatk_gb300 import native

    wl, mapq = _raw_workload(24)
    bad = mapq.copy()
    bad[0] = 300  # the first read of the first region: the first push fails, nothing is queued
    q = engine.raw_queue(wl)
    try:
        with pytest.raises(native.GhmmError, match="mapping quality"):
            q.push_raw(wl, bad)
        got = q.push_raw(wl, mapq)
        q.flush()
    finally:
        q.close()
    assert np.array_equal(got, engine.compute_raw(wl, mapq))


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["standard", "dragstr"])
def test_mirror_computes_from_raw_reads_with_an_imputator(kind):
    # CudaLoglessPairHMM.compute_log10_likelihoods_raw (computeLog10Likelihoods with an input score imputator) on one
    # region's raw reads, against the prepared-planes call on the restatement's planes
    from gatk_gb300.pairhmm import (CudaLoglessPairHMM, DragstrPairHMMInputScoreImputator, PairHMMNativeArguments,
                                    StandardPairHMMInputScoreImputator)

    wl, mapq = _dragstr_workload(31, regions=1)
    imp = DragstrPairHMMInputScoreImputator(*EXAMPLE) if kind == "dragstr" else StandardPairHMMInputScoreImputator(10)
    dragstr = EXAMPLE if kind == "dragstr" else None
    prepared = _prepared_workload(wl, mapq, True, 3.0, dragstr=dragstr)
    reads_raw, reads_prep = [], []
    for r in range(wl.n_reads):
        a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
        reads_raw.append((wl.bases[a:b], wl.quals[a:b], wl.ins[a:b], wl.dels[a:b], int(mapq[r])))
        reads_prep.append((wl.bases[a:b], prepared.quals[a:b], prepared.ins[a:b], prepared.dels[a:b],
                           prepared.gcp[a:b]))
    haps = [wl.hap_bases[int(wl.hap_off[h]):int(wl.hap_off[h + 1])] for h in range(wl.n_haps)]
    with CudaLoglessPairHMM(PairHMMNativeArguments(0, True)) as hmm:
        hmm.initialize(haps)
        got = hmm.compute_log10_likelihoods_raw(reads_raw, imp).copy()
        want = hmm.compute_log10_likelihoods(reads_prep)
    assert np.abs(got - want).max() <= 1e-9


@pytest.mark.parametrize("mode", ["pcr", "pcr_no_tags", "no_pcr", "dragstr"])
def test_c_restatement_matches_the_python_one(mode):
    # oracle/readprep_oracle.c (the large-sample CPU baseline) against oracle/readprep.py, read by read
    from oracle import oracle as O

    wl, mapq = _dragstr_workload(51, regions=2)
    rng = np.random.default_rng(52)
    wl.ins[:] = rng.integers(0, 60, size=len(wl.ins)).astype(np.uint8)
    wl.dels[:] = rng.integers(0, 60, size=len(wl.dels)).astype(np.uint8)
    tags = mode != "pcr_no_tags"
    rate = 0.0 if mode == "no_pcr" else 3.0
    dragstr = EXAMPLE if mode == "dragstr" else None
    q, i, d, g = O.prepare_reads(wl.read_off, wl.bases, wl.quals, wl.ins if tags else None, wl.dels if tags else None,
                                 mapq, rate_factor=rate, dragstr=dragstr)
    want = _prepared_workload(wl, mapq, tags, rate, dragstr=dragstr)
    assert np.array_equal(q, want.quals) and np.array_equal(i, want.ins)
    assert np.array_equal(d, want.dels) and np.array_equal(g, want.gcp)


@pytest.mark.gpu
@pytest.mark.parametrize("kind", ["pcr", "dragstr"])
def test_large_raw_call_is_pipelined_with_identical_results(engine, kind):
    # ghmm_compute_regions_raw on more than 1.5e11 cells runs as a pipeline of batches through the context's queue,
    # each prepared on the device after its upload; a region's results do not depend on the batching
    wl = W.generate(1, regions=1500)
    rng = np.random.default_rng(61)
    wl.quals[:] = rng.integers(2, 45, size=len(wl.quals)).astype(np.uint8)
    mapq = rng.integers(10, 70, size=wl.n_reads)
    assert wl.cells() >= 1.5e11
    kw = {"dragstr": EXAMPLE} if kind == "dragstr" else {"pcr_rate_factor": 3.0}
    got = engine.compute_raw(wl, mapq, **kw)
    with engine.raw_batch(wl, mapq, **kw) as b:
        b.forward()
        want = b.results()
    assert np.array_equal(got, want)
    again = engine.compute(wl)  # a prepared-planes call afterwards runs the same queue without the preparation
    with engine.batch(wl) as b:
        b.forward()
        assert np.array_equal(again, b.results())
