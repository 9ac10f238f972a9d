"""CPU restatement of the step after the likelihoods: normalisation and poorly-modelled-read filtering.

TEST INFRASTRUCTURE ONLY (the oracle for ghmm_batch_postprocess and for the haplotype ghmm_batch_realign
picks).  Plain numpy/Python loops over a
workload's read-major blocks, following (paths inside the GATK repository):

  AlleleLikelihoods.normalizeLikelihoods / normalizeLikelihoodsPerEvidence
      src/main/java/org/broadinstitute/hellbender/utils/genotyper/AlleleLikelihoods.java:416-458
  AlleleLikelihoods.searchBestAllele                                                  :505-560
  AlleleLikelihoods.bestAllelesBreakingTies, BestAllele.isInformative                 :1062-1075, 1269-1282
  AlleleLikelihoods.maximumLikelihoodOverAllAlleles                                   :1198-1208
  AlleleLikelihoods.filterPoorlyModeledEvidence                                       :1351-1376
  ReadLikelihoodCalculationEngine.log10MinTrueLikelihood                              tools/walkers/haplotypecaller/
      ReadLikelihoodCalculationEngine.java:124-132
  ReadLikelihoodCalculationEngine.daynamicLog10MinLiklihoodModel / calculateLog10DynamicReadQualThreshold :106-158
  the dynamic threshold table                                                         :163-182
  PairHMMLikelihoodCalculationEngine.computeReadLikelihoods (normalise, then filter)  :200-201

The alleles of a region are its haplotypes; one region is one sample.
"""
from __future__ import annotations

import math

import numpy as np

# (mean, variance) per base quality 1..40 of the DRAGEN-GATK dynamic read-quality threshold
# (ReadLikelihoodCalculationEngine.java:163-178); a table the product must match value for value.
DYNAMIC_QUAL_TABLE = [
    (5.996842844, 0.196616587), (5.870018422, 1.388545569), (5.401558531, 5.641990128), (4.818940919, 10.33176216),
    (4.218758304, 14.25799688), (3.646319832, 17.02880749), (3.122346753, 18.64537883), (2.654731979, 19.27521677),
    (2.244479156, 19.13584613), (1.88893867, 18.43922003), (1.583645342, 17.36842261), (1.3233807, 16.07088712),
    (1.102785365, 14.65952563), (0.916703025, 13.21718577), (0.760361881, 11.80207947), (0.629457387, 10.45304833),
    (0.520175654, 9.194183767), (0.42918208, 8.038657241), (0.353590663, 6.991779595), (0.290923699, 6.053379213),
    (0.23906788, 5.219610436), (0.196230431, 4.484302033), (0.160897421, 3.839943445), (0.131795374, 3.27839108),
    (0.1078567, 2.791361596), (0.088189063, 2.370765375), (0.072048567, 2.008921719), (0.058816518, 1.698687797),
    (0.047979438, 1.433525748), (0.039111985, 1.207526336), (0.031862437, 1.015402928), (0.025940415, 0.852465956),
    (0.021106532, 0.714585285), (0.017163711, 0.598145851), (0.013949904, 0.500000349), (0.011332027, 0.41742159),
    (0.009200898, 0.348056286), (0.007467036, 0.289881373), (0.006057179, 0.241163527), (0.004911394, 0.200422214),
]


def best_allele(values, reference: int, can_be_reference: bool) -> float:
    """searchBestAllele's likelihood (AlleleLikelihoods.java:505-540); -inf when there is no candidate."""
    n = len(values)
    if n == 0 or (n == 1 and reference == 0 and not can_be_reference):
        return -math.inf
    best_index = 0 if (can_be_reference or reference != 0) else 1
    best = values[best_index]
    for a in range(best_index + 1, n):
        if not can_be_reference and reference == a:
            continue
        if values[a] > best:
            best = values[a]
    return best


LOG_10_INFORMATIVE_THRESHOLD = 0.2  # AlleleLikelihoods.java:38


def best_allele_breaking_ties(values, priorities=None):
    """searchBestAllele(sample, read, canBeReference = true, priorities) (AlleleLikelihoods.java:505-560) as
    bestAllelesBreakingTies calls it (:1062-1075): (best index, BestAllele.isInformative() (:1269-1282))."""
    n = len(values)
    if n == 0:
        return -1, False
    best, second = 0, 0
    best_l, second_l = values[0], -math.inf
    for a in range(1, n):
        c = values[a]
        if c > best_l:
            second, best, second_l, best_l = best, a, best_l, c
        elif c > second_l:
            second, second_l = a, c
    thr = LOG_10_INFORMATIVE_THRESHOLD
    if priorities is not None and best_l - second_l < thr:
        best_p, second_p = priorities[best], priorities[second]
        for a in range(n):
            c = values[a]
            if a == best or best_l - c > thr:
                continue
            cp = priorities[a]
            if cp > best_p:
                second, best, second_p, best_p = best, a, best_p, cp
            elif cp > second_p:
                second, second_p = a, cp
    best_l = values[best]
    second_l = values[second] if second != best else -math.inf
    confidence = 0.0 if best_l == second_l else best_l - second_l
    return best, confidence > thr


def min_true_likelihood(read_len: int, rate: float, cap: bool) -> float:
    """log10MinTrueLikelihood (ReadLikelihoodCalculationEngine.java:124-132)."""
    max_errors = min(2.0, math.ceil(read_len * rate)) if cap else math.ceil(read_len * rate)
    return max_errors * -4.0


def dynamic_threshold(quals, scale: float) -> float:
    """calculateLog10DynamicReadQualThreshold (ReadLikelihoodCalculationEngine.java:137-158)."""
    s_mean = 0.0
    s_var = 0.0
    for q in quals:
        bq = int(q) & 0xFF
        e = 0 if bq <= 1 else min(40, bq) - 1
        s_mean += DYNAMIC_QUAL_TABLE[e][0]
        s_var += DYNAMIC_QUAL_TABLE[e][1]
    return (s_mean + scale * math.sqrt(s_var)) * -0.1


def read_threshold(quals, rate: float, dynamic: bool, scale: float) -> float:
    """The filter threshold of one read (ReadLikelihoodCalculationEngine.java:98-119)."""
    if dynamic:
        d = dynamic_threshold(quals, scale)
        m = min_true_likelihood(len(quals), rate, False)
        return d if d < m else m
    return min_true_likelihood(len(quals), rate, True)


def postprocess(wl, out: np.ndarray, cap: float, symmetric: bool, reference=None, rate: float = 0.02,
                dynamic: bool = False, scale: float = 1.0):
    """Normalise `out` (a workload's read-major blocks) and flag the reads to keep.

    cap: log10globalReadMismappingRate (< 0, or -inf to skip normalisation); symmetric: the best allele may be
    the reference; reference: per region, the reference haplotype's index within the region (or -1).
    Returns (normalised copy of out, keep flags per read as uint8).
    """
    vals = np.array(out, dtype=np.float64, copy=True)
    keep = np.ones(wl.n_reads, dtype=np.uint8)
    for g in range(wl.n_regions):
        r0, r1 = int(wl.region_read_off[g]), int(wl.region_read_off[g + 1])
        nh = int(wl.region_hap_off[g + 1] - wl.region_hap_off[g])
        o = int(wl.out_off[g])
        ref = -1 if reference is None else int(reference[g])
        for k, r in enumerate(range(r0, r1)):
            row = vals[o + k * nh: o + (k + 1) * nh]
            if cap != -math.inf and nh > 1:
                b = best_allele(row, ref, symmetric)
                worst = b + cap
                for a in range(nh):
                    if row[a] < worst:
                        row[a] = worst
            mx = -math.inf
            for a in range(nh):
                if row[a] > mx:
                    mx = row[a]
            q = wl.quals[int(wl.read_off[r]):int(wl.read_off[r + 1])]
            if mx < read_threshold(q, rate, dynamic, scale):
                keep[r] = 0
    return vals, keep
