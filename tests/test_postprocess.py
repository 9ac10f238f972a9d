"""The step after the likelihoods: normalisation (AlleleLikelihoods.normalizeLikelihoods) and the
poorly-modelled-read filter (filterPoorlyModeledEvidence), on the device against the CPU restatement
oracle/postprocess.py.  The arithmetic is IEEE double with no contraction on both sides, so the comparison is
exact."""
import math

import numpy as np
import pytest

from gatk_gb300 import workload as W
from oracle import oracle as O
from oracle import postprocess as P


def _random_matrix(rng, wl):
    return -rng.gamma(2.0, 6.0, size=wl.n_pairs)


def test_normalise_matches_the_reference_known_answer_rule():
    # AlleleLikelihoodsUnitTest.testNormalizeCapWorstLK: with symmetric normalisation every likelihood becomes
    # max(original, best - cap), and rows whose best is -inf stay as they are
    rng = np.random.default_rng(2)
    wl = W.generate(1, regions=5)
    out = _random_matrix(rng, wl)
    out[: int(wl.out_off[1])] = -np.inf  # first region: all -inf
    vals, _ = P.postprocess(wl, out, -0.001, True)
    for g in range(wl.n_regions):
        nh = int(wl.region_hap_off[g + 1] - wl.region_hap_off[g])
        o = int(wl.out_off[g])
        for k in range(int(wl.region_read_off[g + 1] - wl.region_read_off[g])):
            row, new = out[o + k * nh:o + (k + 1) * nh], vals[o + k * nh:o + (k + 1) * nh]
            best = row.max()
            if best == -np.inf or nh <= 1:
                assert np.array_equal(new, row)
            else:
                assert np.array_equal(new, np.maximum(row, best - 0.001))


def test_best_allele_excludes_the_reference_when_asymmetric():
    row = np.array([-1.0, -5.0, -3.0])
    assert P.best_allele(row, 0, True) == -1.0
    assert P.best_allele(row, 0, False) == -3.0
    assert P.best_allele(row, 2, False) == -1.0
    assert P.best_allele(np.array([-2.0]), 0, False) == -math.inf


def test_thresholds():
    # log10MinTrueLikelihood: min(2, ceil(L * rate)) errors of -4 each (capped), ceil(L * rate) uncapped
    assert P.min_true_likelihood(150, 0.02, True) == -8.0
    assert P.min_true_likelihood(40, 0.02, True) == -4.0
    assert P.min_true_likelihood(150, 0.02, False) == -12.0
    # dynamic: sum of per-quality means + K sqrt(sum of variances), times -0.1
    q = np.full(100, 30, dtype=np.uint8)
    mean, var = P.DYNAMIC_QUAL_TABLE[29]
    assert P.dynamic_threshold(q, 1.0) == (100 * mean + math.sqrt(100 * var)) * -0.1 or \
        abs(P.dynamic_threshold(q, 1.0) - (100 * mean + math.sqrt(100 * var)) * -0.1) < 1e-12
    assert len(P.DYNAMIC_QUAL_TABLE) == 40


@pytest.mark.gpu
@pytest.mark.parametrize("cap,symmetric,dynamic,use_ref", [(-4.5, True, False, False), (-4.5, False, False, True),
                                                           (-2.0, True, True, True), (-math.inf, True, False, False),
                                                           (-0.001, False, True, False)])
def test_device_postprocess_matches_oracle(engine, cap, symmetric, dynamic, use_ref):
    wl = W.generate(1, regions=40)
    rng = np.random.default_rng(9)
    ref = rng.integers(-1, 3, size=wl.n_regions).astype(np.int32) if use_ref else None
    if ref is not None:
        nh = np.diff(wl.region_hap_off)
        ref = np.where(ref < nh, ref, -1).astype(np.int32)
    with engine.batch(wl) as b:
        b.forward()
        raw = b.results()
        keep = b.postprocess(cap=cap, symmetric=symmetric, reference_hap=ref, dynamic=dynamic, scale=1.0)
        got = b.results()
    want, want_keep = P.postprocess(wl, raw, cap, symmetric, ref, 0.02, dynamic, 1.0)
    assert np.array_equal(got, want)
    assert np.array_equal(keep, want_keep)
    assert keep.shape == (wl.n_reads,)
