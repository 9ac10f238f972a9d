/*
 * pdhmm_oracle.c -- FP64 CPU oracle for the partially-determined-haplotype PairHMM (PD-HMM).
 *
 * TEST INFRASTRUCTURE ONLY: linked by the tests and the cpu_baseline leg of bench.py, never by the
 * product library.  Strict IEEE double arithmetic (-ffp-contract=off), Java's operation order.
 *
 * It restates (paths inside the GATK repository):
 *   LoglessPDPairHMM.subComputeReadLikelihoodGivenHaplotypeLog10
 *       src/main/java/org/broadinstitute/hellbender/utils/pairhmm/LoglessPDPairHMM.java:35-150
 *   LoglessPDPairHMM.initializePriors / isBasePDMatching                                :176-210
 *   PartiallyDeterminedHaplotype flag bits (SNP 1, DEL_START 2, DEL_END 4, A 8, C 16, G 32, T 64, N 128)
 *       src/main/java/org/broadinstitute/hellbender/utils/haplotype/PartiallyDeterminedHaplotype.java:59-66
 * with the transition model of pairhmm_oracle.c (PairHMMModel.qualToTransProbs).
 *
 * The computation starts at haplotype column 1 for every pair: PDPairHMM.computeReadLikelihoodGivenHaplotypeLog10
 * disables the cross-haplotype prefix reuse (nextHapStartIndex = 0, PDPairHMM.java:286-288).  The HMM state
 * (NORMAL / INSIDE_DEL / AFTER_DEL) lives outside the row loop in the reference, so a row starts in the state the
 * previous row ended in; this restatement keeps that.
 *
 * Parity: the reference's PD-HMM golden file (src/test/resources/large/expected.PDHMM.hmmresults.txt) is a git-lfs
 * pointer in this checkout, so this oracle is "parity unpinned" against the reference's own outputs.  It is pinned
 * to the plain oracle instead: with no PD flags the recurrence is LoglessPairHMM's, and the tests check that the two
 * agree bit for bit.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

#ifdef _OPENMP
#include <omp.h>
#endif

void oracle_qual_to_trans_probs(double dest[6], int ins, int del, int gcp);
double oracle_qual_to_error_prob(int q);
double oracle_qual_to_prob(int q);
double oracle_initial_condition_log10(void);

enum { PD_MM = 0, PD_IM = 1, PD_MI = 2, PD_II = 3, PD_MD = 4, PD_DD = 5 };
enum { PD_SNP = 1, PD_DEL_START = 2, PD_DEL_END = 4, PD_A = 8, PD_C = 16, PD_G = 32, PD_T = 64 };
enum { ST_NORMAL = 0, ST_INSIDE_DEL = 1, ST_AFTER_DEL = 2 };

static double jmax(double a, double b) { return (a >= b) ? a : b; } /* Math.max for the non-NaN values here */

/* isBasePDMatching (LoglessPDPairHMM.java:196-210); *bad set where the reference throws */
static int pd_matching(uint8_t x, uint8_t pd, int *bad) {
    if (pd & PD_SNP) {
        switch (x) {
            case 'A': case 'a': return (pd & PD_A) != 0;
            case 'C': case 'c': return (pd & PD_C) != 0;
            case 'T': case 't': return (pd & PD_T) != 0;
            case 'G': case 'g': return (pd & PD_G) != 0;
            default: *bad = 1; return 0;
        }
    }
    return 0;
}

/*
 * log10 likelihood of one read against one partially determined haplotype.  *err = 1 where the reference throws
 * ("Found unexpected base in alt alleles"); the return value is then NaN.
 */
double oracle_pd_logless(const uint8_t *hap, const uint8_t *pd, int H, const uint8_t *rb, const uint8_t *q,
                         const uint8_t *ins, const uint8_t *del, const uint8_t *gcp, int R, int *err) {
    *err = 0;
    const size_t W = (size_t)H + 1;
    double *buf = (double *)calloc(12 * W, sizeof(double));
    double *pM = buf, *pI = buf + W, *pD = buf + 2 * W, *pbM = buf + 3 * W, *pbI = buf + 4 * W, *pbD = buf + 5 * W;
    double *cM = buf + 6 * W, *cI = buf + 7 * W, *cD = buf + 8 * W, *cbM = buf + 9 * W, *cbI = buf + 10 * W,
           *cbD = buf + 11 * W;
    const double initial = ldexp(1.0, 1020) / (double)H;
    for (int j = 0; j <= H; j++) pD[j] = initial; /* row 0: D = 2^1020 / H, everything else 0 */
    int state = ST_NORMAL;
    for (int i = 1; i <= R; i++) {
        double t[6];
        oracle_qual_to_trans_probs(t, ins[i - 1], del[i - 1], gcp[i - 1]);
        const uint8_t x = rb[i - 1];
        const double p_match = oracle_qual_to_prob(q[i - 1]);
        const double p_mis = oracle_qual_to_error_prob(q[i - 1]) / 3.0;
        cM[0] = cI[0] = cD[0] = 0.0; /* column 0 is never written by the reference: zeros */
        cbM[0] = cbI[0] = cbD[0] = 0.0;
        for (int j = 1; j <= H; j++) {
            const uint8_t y = hap[j - 1], f = pd[j - 1];
            int bad = 0;
            const int m = (x == y || x == 'N' || y == 'N' || pd_matching(x, f, &bad));
            if (bad) {
                *err = 1;
                free(buf);
                return NAN;
            }
            const double prior = m ? p_match : p_mis;
            const int del_end_here = (f & PD_DEL_END) == PD_DEL_END;
            switch (state) {
                case ST_NORMAL:
                case ST_INSIDE_DEL:
                    if (state == ST_NORMAL) {
                        cbM[j] = cM[j - 1];
                        cbD[j] = cD[j - 1];
                        cbI[j] = cI[j - 1];
                    } else {
                        cbM[j] = cbM[j - 1];
                        cbD[j] = cbD[j - 1];
                        cbI[j] = cbI[j - 1];
                    }
                    cM[j] = prior * (pM[j - 1] * t[PD_MM] + pI[j - 1] * t[PD_IM] + pD[j - 1] * t[PD_IM]);
                    cD[j] = cM[j - 1] * t[PD_MD] + cD[j - 1] * t[PD_DD];
                    break;
                default: /* ST_AFTER_DEL */
                    cbM[j] = jmax(cbM[j - 1], cM[j - 1]);
                    cbD[j] = jmax(cbD[j - 1], cD[j - 1]);
                    cbI[j] = jmax(cbI[j - 1], cI[j - 1]);
                    cM[j] = prior * (jmax(pbM[j - 1], pM[j - 1]) * t[PD_MM] + jmax(pbI[j - 1], pI[j - 1]) * t[PD_IM] +
                                     jmax(pbD[j - 1], pD[j - 1]) * t[PD_IM]);
                    cD[j] = jmax(cbM[j - 1], cM[j - 1]) * t[PD_MD] + jmax(cbD[j - 1], cD[j - 1]) * t[PD_DD];
                    break;
            }
            if (del_end_here)
                cI[j] = jmax(pbM[j], pM[j]) * t[PD_MI] + jmax(pbI[j], pI[j]) * t[PD_II];
            else
                cI[j] = pM[j] * t[PD_MI] + pI[j] * t[PD_II];
            if (state == ST_AFTER_DEL) state = ST_NORMAL;
            if ((f & PD_DEL_START) == PD_DEL_START) state = ST_INSIDE_DEL;
            if ((f & PD_DEL_END) == PD_DEL_END) state = ST_AFTER_DEL;
        }
        double *s;
        s = pM; pM = cM; cM = s;
        s = pI; pI = cI; cI = s;
        s = pD; pD = cD; cD = s;
        s = pbM; pbM = cbM; cbM = s;
        s = pbI; pbI = cbI; cbI = s;
        s = pbD; pbD = cbD; cbD = s;
    }
    double sum = 0.0;
    if (R > 0)
        for (int j = 1; j <= H; j++) sum += pM[j] + pI[j];
    free(buf);
    return log10(sum) - oracle_initial_condition_log10();
}

/* Every (read, haplotype) pair of a flat PD workload, read-major per region; OpenMP over pairs.  Returns the
 * number of pairs where the reference throws (their slot holds NaN). */
int64_t oracle_pd_compute_pairs(int64_t n_pairs, const int64_t *pair_read, const int64_t *pair_hap,
                                const int64_t *read_off, const uint8_t *bases, const uint8_t *quals,
                                const uint8_t *ins, const uint8_t *del, const uint8_t *gcp, const int64_t *hap_off,
                                const uint8_t *hap, const uint8_t *pd, double *out, int threads) {
    int64_t bad = 0;
#ifdef _OPENMP
    omp_set_num_threads(threads > 0 ? threads : omp_get_num_procs());
#endif
#pragma omp parallel for schedule(dynamic, 16) reduction(+ : bad)
    for (int64_t p = 0; p < n_pairs; p++) {
        const int64_t r = pair_read[p], h = pair_hap[p];
        const int64_t a = read_off[r], b = read_off[r + 1], c = hap_off[h], d = hap_off[h + 1];
        int err = 0;
        out[p] = oracle_pd_logless(hap + c, pd + c, (int)(d - c), bases + a, quals + a, ins + a, del + a, gcp + a,
                                   (int)(b - a), &err);
        bad += err;
    }
    return bad;
}
