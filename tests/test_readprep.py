"""Read preparation before the PairHMM (PairHMMLikelihoodCalculationEngine.modifyReadQualities, the PCR indel
error model with findTandemRepeatUnits, standard imputation): the CPU restatement oracle/readprep.py against the
reference's own unit-test cases, and the device path (ghmm_compute_regions_raw) against the regular forward on
the restatement's prepared planes (identical planes give identical results)."""
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


def _prepared_workload(wl, mapq, with_indel, rate, threshold=18, cap=True, gcp=10):
    planes = [np.empty_like(wl.bases) for _ in range(4)]
    for r in range(wl.n_reads):
        a, b = int(wl.read_off[r]), int(wl.read_off[r + 1])
        _, q, i, d, g = RP.prepare_read(wl.bases[a:b], wl.quals[a:b], wl.ins[a:b] if with_indel else None,
                                        wl.dels[a:b] if with_indel else None, int(mapq[r]), threshold, cap, rate, gcp)
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
