/*
 * pairhmm_oracle.c -- FP64 CPU oracle for the GATK PairHMM read-likelihood path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: it is linked by the tests,
 * by __graft_entry__.smoke() and by the cpu_baseline / --impl reference leg of
 * bench.py, never by the product library (gatk_gb300/csrc).  The product must not
 * import, call or link anything built from here.
 *
 * It restates, in plain C with strict IEEE double arithmetic (built with
 * -ffp-contract=off so no multiply-add is fused, matching Java semantics), the
 * reference algorithms:
 *
 *   QualityUtils          src/main/java/org/broadinstitute/hellbender/utils/QualityUtils.java:37-57,83-85,138-158,174-190
 *   JacobianLogTable      src/main/java/org/broadinstitute/hellbender/utils/MathUtils.java:406-430,467-480
 *   log10SumLog10 (exact) src/main/java/org/broadinstitute/hellbender/utils/MathUtils.java:622-646
 *   PairHMMModel          src/main/java/org/broadinstitute/hellbender/utils/pairhmm/PairHMMModel.java:86-117,214-225,373-418
 *   LoglessPairHMM        src/main/java/org/broadinstitute/hellbender/utils/pairhmm/LoglessPairHMM.java:8-104
 *   Log10PairHMM          src/main/java/org/broadinstitute/hellbender/utils/pairhmm/Log10PairHMM.java:44-183
 *   PairHMM validation    src/main/java/org/broadinstitute/hellbender/utils/pairhmm/PairHMM.java:275-316
 *
 * Parity pin: expected.Java.hmmresults.txt (284 pairs, printed %e) and
 * pairhmm-testdata.txt (104 pairs, 1e-5) from the reference test resources; see
 * tests/test_oracle_golden.py.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_MAX_QUAL 254                       /* QualityUtils.java:43 */
#define OR_JAC_MAX_TOLERANCE 8.0              /* MathUtils.java:409 */
#define OR_JAC_TABLE_STEP 0.0001              /* MathUtils.java:414 */
#define OR_M2M_SIZE (((OR_MAX_QUAL + 1) * (OR_MAX_QUAL + 2)) >> 1)

enum { OR_MM = 0, OR_IM = 1, OR_MI = 2, OR_II = 3, OR_MD = 4, OR_DD = 5 }; /* PairHMMModel.java:26-51 */

static double or_qual_err[OR_MAX_QUAL + 1];       /* qualToErrorProbCache */
static double or_qual_prob_log10[OR_MAX_QUAL + 1]; /* qualToProbLog10Cache */
static double *or_jacobian = NULL;                 /* JacobianLogTable.cache */
static int or_jacobian_n = 0;
static double or_m2m_prob[OR_M2M_SIZE];
static double or_m2m_log10[OR_M2M_SIZE];
static double or_inv_step;
static double or_initial_condition;       /* 2^1020, LoglessPairHMM.java:8 */
static double or_initial_condition_log10; /* LoglessPairHMM.java:9 */
static double or_log10_3;                 /* Log10PairHMM.java:21 */

/* MathUtils.fastRound, MathUtils.java:428-430 */
static int or_fast_round(double d) { return (d > 0.0) ? (int)(d + 0.5) : (int)(d - 0.5); }

static double or_jacobian_get(double diff) { return or_jacobian[or_fast_round(diff * or_inv_step)]; }

/* MathUtils.approximateLog10SumLog10(double, double), MathUtils.java:467-480 */
double oracle_approx_log10_sum_log10(double a, double b) {
    if (a > b) return oracle_approx_log10_sum_log10(b, a);
    if (a == -INFINITY) return b;
    const double diff = b - a;
    return b + (diff < OR_JAC_MAX_TOLERANCE ? or_jacobian_get(diff) : 0.0);
}

__attribute__((constructor)) static void or_init_tables(void) {
    /* QualityUtils static block, QualityUtils.java:52-57 */
    for (int i = 0; i <= OR_MAX_QUAL; i++) {
        or_qual_err[i] = pow(10.0, ((double)i) / -10.0);
        or_qual_prob_log10[i] = log10(1.0 - or_qual_err[i]);
    }
    /* JacobianLogTable, MathUtils.java:414-418: IndexRange(0, (int)(8/step) + 1) */
    or_inv_step = 1.0 / OR_JAC_TABLE_STEP;
    or_jacobian_n = (int)(OR_JAC_MAX_TOLERANCE / OR_JAC_TABLE_STEP) + 1;
    or_jacobian = (double *)malloc(sizeof(double) * (size_t)or_jacobian_n);
    for (int k = 0; k < or_jacobian_n; k++)
        or_jacobian[k] = log10(1.0 + pow(10.0, -((double)k) * OR_JAC_TABLE_STEP));
    /* PairHMMModel static block, PairHMMModel.java:86-94 */
    const double inv_ln10 = 1.0 / log(10.0);
    for (int i = 0, offset = 0; i <= OR_MAX_QUAL; offset += ++i)
        for (int j = 0; j <= i; j++) {
            const double log10_sum = oracle_approx_log10_sum_log10(-0.1 * i, -0.1 * j);
            double p = pow(10.0, log10_sum);
            if (p > 1.0) p = 1.0;
            or_m2m_log10[offset + j] = log1p(-p) * inv_ln10;
            or_m2m_prob[offset + j] = pow(10.0, or_m2m_log10[offset + j]);
        }
    or_initial_condition = ldexp(1.0, 1020);
    or_initial_condition_log10 = log10(or_initial_condition);
    or_log10_3 = log10(3.0);
}

/* QualityUtils.qualToErrorProb(byte), QualityUtils.java:156-158 (index = qual & 0xFF) */
double oracle_qual_to_error_prob(int q) { return or_qual_err[q & 0xFF]; }
/* QualityUtils.qualToProb(byte), QualityUtils.java:83-85 */
double oracle_qual_to_prob(int q) { return 1.0 - or_qual_err[q & 0xFF]; }

/* PairHMMModel.matchToMatchProb(int,int), PairHMMModel.java:373-388 */
double oracle_match_to_match_prob(int ins, int del) {
    const int mn = ins <= del ? ins : del;
    const int mx = ins <= del ? del : ins;
    if (OR_MAX_QUAL < mx)
        return 1.0 - pow(10.0, oracle_approx_log10_sum_log10(-0.1 * mn, -0.1 * mx));
    return or_m2m_prob[((mx * (mx + 1)) >> 1) + mn];
}

/* PairHMMModel.matchToMatchProbLog10(int,int), PairHMMModel.java:404-418 */
double oracle_match_to_match_prob_log10(int ins, int del) {
    const int mn = ins <= del ? ins : del;
    const int mx = ins <= del ? del : ins;
    if (OR_MAX_QUAL < mx) {
        double p = pow(10.0, oracle_approx_log10_sum_log10(-0.1 * mn, -0.1 * mx));
        if (p > 1.0) p = 1.0;
        return log1p(-p) * (1.0 / log(10.0));
    }
    return or_m2m_log10[((mx * (mx + 1)) >> 1) + mn];
}

/* PairHMMModel.qualToTransProbs(double[],byte,byte,byte), PairHMMModel.java:107-117 */
void oracle_qual_to_trans_probs(double dest[6], int ins, int del, int gcp) {
    dest[OR_MM] = oracle_match_to_match_prob(ins, del);
    dest[OR_MI] = oracle_qual_to_error_prob(ins);
    dest[OR_MD] = oracle_qual_to_error_prob(del);
    dest[OR_IM] = oracle_qual_to_prob(gcp);
    dest[OR_II] = dest[OR_DD] = oracle_qual_to_error_prob(gcp);
}

/* PairHMMModel.qualToTransProbsLog10, PairHMMModel.java:214-225 */
void oracle_qual_to_trans_probs_log10(double dest[6], int ins, int del, int gcp) {
    dest[OR_MM] = oracle_match_to_match_prob_log10(ins, del);
    dest[OR_MI] = (double)(ins & 0xFF) * -0.1;
    dest[OR_MD] = (double)(del & 0xFF) * -0.1;
    dest[OR_IM] = or_qual_prob_log10[gcp & 0xFF];
    dest[OR_II] = (double)(gcp & 0xFF) * -0.1;
    dest[OR_DD] = (double)(gcp & 0xFF) * -0.1;
}

/*
 * Validation mirrored from PairHMMModel.qualToTransProbs (ins/del/gcp >= 0 as Java
 * signed bytes, PairHMMModel.java:109-111) and QualityUtils' cache size (base quality
 * byte & 0xFF must index a 255-entry cache, QualityUtils.java:48-57).
 * Returns 0 if valid, -1 otherwise.
 */
int oracle_validate_read(const uint8_t *q, const uint8_t *ins, const uint8_t *del, const uint8_t *gcp, int R) {
    for (int i = 0; i < R; i++) {
        if (q[i] > OR_MAX_QUAL) return -1;
        if (ins[i] > 127 || del[i] > 127 || gcp[i] > 127) return -1;
    }
    return 0;
}

static int or_is_match(uint8_t x, uint8_t y) { return x == y || x == (uint8_t)'N' || y == (uint8_t)'N'; }

/*
 * LoglessPairHMM.subComputeReadLikelihoodGivenHaplotypeLog10 (LoglessPairHMM.java:20-68)
 * with initializePriors (:79-93) and initializeProbabilities (:102-104), evaluated
 * with two rolling rows instead of full matrices (identical arithmetic).
 */
double oracle_logless(const uint8_t *hap, int H, const uint8_t *rb, const uint8_t *q, const uint8_t *ins,
                      const uint8_t *del, const uint8_t *gcp, int R, int tristate) {
    const double tri = tristate ? 3.0 : 1.0;
    double *buf = (double *)calloc((size_t)6 * (size_t)(H + 1), sizeof(double));
    double *Mp = buf, *Ip = buf + (H + 1), *Dp = buf + 2 * (H + 1);
    double *Mc = buf + 3 * (H + 1), *Ic = buf + 4 * (H + 1), *Dc = buf + 5 * (H + 1);
    const double initial = or_initial_condition / (double)H;
    for (int j = 0; j <= H; j++) Dp[j] = initial;
    for (int i = 1; i <= R; i++) {
        double t[6];
        oracle_qual_to_trans_probs(t, ins[i - 1], del[i - 1], gcp[i - 1]);
        const double p_match = oracle_qual_to_prob(q[i - 1]);
        const double p_mis = oracle_qual_to_error_prob(q[i - 1]) / tri;
        Mc[0] = 0.0;
        Ic[0] = 0.0;
        Dc[0] = 0.0;
        for (int j = 1; j <= H; j++) {
            const double prior = or_is_match(rb[i - 1], hap[j - 1]) ? p_match : p_mis;
            Mc[j] = prior * (Mp[j - 1] * t[OR_MM] + Ip[j - 1] * t[OR_IM] + Dp[j - 1] * t[OR_IM]);
            Ic[j] = Mp[j] * t[OR_MI] + Ip[j] * t[OR_II];
            Dc[j] = Mc[j - 1] * t[OR_MD] + Dc[j - 1] * t[OR_DD];
        }
        double *s;
        s = Mp; Mp = Mc; Mc = s;
        s = Ip; Ip = Ic; Ic = s;
        s = Dp; Dp = Dc; Dc = s;
    }
    /* Final sum over M and I of the last row only (LoglessPairHMM.java:62-67); with R == 0
     * the last row is row 0, whose M and I are zero. */
    double sum = 0.0;
    if (R == 0) {
        sum = 0.0;
    } else {
        for (int j = 1; j <= H; j++) sum += Mp[j] + Ip[j];
    }
    free(buf);
    return log10(sum) - or_initial_condition_log10;
}

/* MathUtils.log10SumLog10(double[]) (exact), MathUtils.java:622-646 */
static double or_log10_sum_exact(const double *v, int n) {
    if (n <= 0) return -INFINITY;
    int mi = 0;
    for (int i = 1; i < n; i++)
        if (v[i] > v[mi]) mi = i;
    const double mx = v[mi];
    if (mx == -INFINITY) return mx;
    double sum = 1.0;
    for (int i = 0; i < n; i++) {
        if (i == mi || v[i] == -INFINITY) continue;
        sum += pow(10.0, v[i] - mx);
    }
    return mx + (sum != 1.0 ? log10(sum) : 0.0);
}

/* MathUtils.approximateLog10SumLog10(double[], int), MathUtils.java:444-460 */
static double or_log10_sum_approx(const double *v, int n) {
    int mi = 0;
    for (int i = 1; i < n; i++)
        if (v[i] > v[mi]) mi = i;
    double s = v[mi];
    for (int i = 0; i < n; i++) {
        if (i == mi || v[i] == -INFINITY) continue;
        const double diff = s - v[i];
        s += diff < OR_JAC_MAX_TOLERANCE ? or_jacobian_get(diff) : 0.0;
    }
    return s;
}

static double or_lsum(const double *v, int n, int exact) {
    return exact ? or_log10_sum_exact(v, n) : or_log10_sum_approx(v, n);
}

/*
 * Log10PairHMM.subComputeReadLikelihoodGivenHaplotypeLog10 (Log10PairHMM.java:58-105),
 * updateCell (:175-183), initializeLog10Priors (:117-131); exact = EXACT, !exact = ORIGINAL.
 */
double oracle_log10_hmm(const uint8_t *hap, int H, const uint8_t *rb, const uint8_t *q, const uint8_t *ins,
                        const uint8_t *del, const uint8_t *gcp, int R, int tristate, int exact) {
    double *buf = (double *)malloc(sizeof(double) * (size_t)6 * (size_t)(H + 1));
    double *Mp = buf, *Ip = buf + (H + 1), *Dp = buf + 2 * (H + 1);
    double *Mc = buf + 3 * (H + 1), *Ic = buf + 4 * (H + 1), *Dc = buf + 5 * (H + 1);
    for (int j = 0; j <= H; j++) {
        Mp[j] = -INFINITY;
        Ip[j] = -INFINITY;
        Dp[j] = log10(1.0 / (double)H);
    }
    for (int i = 1; i <= R; i++) {
        double t[6];
        oracle_qual_to_trans_probs_log10(t, ins[i - 1], del[i - 1], gcp[i - 1]);
        const double p_match = or_qual_prob_log10[q[i - 1] & 0xFF];
        const double p_mis = (double)(q[i - 1] & 0xFF) * -0.1 - (tristate ? or_log10_3 : 0.0);
        Mc[0] = -INFINITY;
        Ic[0] = -INFINITY;
        Dc[0] = -INFINITY;
        for (int j = 1; j <= H; j++) {
            const double prior = or_is_match(rb[i - 1], hap[j - 1]) ? p_match : p_mis;
            double v3[3] = {Mp[j - 1] + t[OR_MM], Ip[j - 1] + t[OR_IM], Dp[j - 1] + t[OR_IM]};
            Mc[j] = prior + or_lsum(v3, 3, exact);
            double v2[2] = {Mp[j] + t[OR_MI], Ip[j] + t[OR_II]};
            Ic[j] = or_lsum(v2, 2, exact);
            double w2[2] = {Mc[j - 1] + t[OR_MD], Dc[j - 1] + t[OR_DD]};
            Dc[j] = or_lsum(w2, 2, exact);
        }
        double *s;
        s = Mp; Mp = Mc; Mc = s;
        s = Ip; Ip = Ic; Ic = s;
        s = Dp; Dp = Dc; Dc = s;
    }
    /* finalLog10LikelihoodCalculation, Log10PairHMM.java:98-105 */
    double acc;
    {
        double v[2] = {Mp[1], Ip[1]};
        acc = or_lsum(v, 2, exact);
    }
    for (int j = 2; j <= H; j++) {
        double v[3] = {acc, Mp[j], Ip[j]};
        acc = or_lsum(v, 3, exact);
    }
    free(buf);
    return acc;
}

/*
 * Batched evaluation over a flat workload, as the reference's PairHMM.computeLog10Likelihoods
 * (PairHMM.java:196-247) does per region: for each region, for each read r and haplotype a,
 * out[out_off[region] + r * n_haps + a] (read-major, VectorLoglessPairHMM.java:131,147).
 *
 *   region_read_off[n_regions+1], region_hap_off[n_regions+1]: index ranges into reads/haps
 *   read_off[n_reads+1]: byte offset of each read in the five planes (bases, quals, ins, del, gcp)
 *   hap_off[n_haps+1]: byte offset of each haplotype in hap_bases
 *   out_off[n_regions+1]: offsets into out
 *
 * threads <= 0 uses all OpenMP threads.  Returns the number of pairs evaluated.
 */
int64_t oracle_compute_regions(int32_t n_regions, const int64_t *region_read_off, const int64_t *region_hap_off,
                               const int64_t *read_off, const uint8_t *bases, const uint8_t *quals,
                               const uint8_t *ins, const uint8_t *del, const uint8_t *gcp, const int64_t *hap_off,
                               const uint8_t *hap_bases, const int64_t *out_off, double *out, int threads) {
    int64_t total = 0;
    for (int32_t g = 0; g < n_regions; g++)
        total += (region_read_off[g + 1] - region_read_off[g]) * (region_hap_off[g + 1] - region_hap_off[g]);
#ifdef _OPENMP
    omp_set_num_threads(threads > 0 ? threads : omp_get_num_procs());
#else
    (void)threads;
#endif
    for (int32_t g = 0; g < n_regions; g++) {
        const int64_t r0 = region_read_off[g], nr = region_read_off[g + 1] - r0;
        const int64_t h0 = region_hap_off[g], nh = region_hap_off[g + 1] - h0;
        const int64_t npairs = nr * nh;
#pragma omp parallel for schedule(dynamic, 4)
        for (int64_t p = 0; p < npairs; p++) {
            const int64_t r = r0 + p / nh, h = h0 + p % nh;
            const int64_t o = read_off[r];
            const int R = (int)(read_off[r + 1] - o);
            const int H = (int)(hap_off[h + 1] - hap_off[h]);
            out[out_off[g] + p] = oracle_logless(hap_bases + hap_off[h], H, bases + o, quals + o, ins + o, del + o,
                                                 gcp + o, R, 1);
        }
    }
    return total;
}

/* Table accessors used by the tests to check the product's tables element by element. */
int oracle_jacobian_size(void) { return or_jacobian_n; }
double oracle_jacobian_value(int k) { return (k >= 0 && k < or_jacobian_n) ? or_jacobian[k] : NAN; }
double oracle_initial_condition_log10(void) { return or_initial_condition_log10; }

/* Parallel map over pairs given by explicit index lists (used for subsample parity). */
void oracle_compute_pairs(int64_t n_pairs, const int64_t *pair_read, const int64_t *pair_hap, const int64_t *read_off,
                          const uint8_t *bases, const uint8_t *quals, const uint8_t *ins, const uint8_t *del,
                          const uint8_t *gcp, const int64_t *hap_off, const uint8_t *hap_bases, double *out,
                          int threads) {
#ifdef _OPENMP
    omp_set_num_threads(threads > 0 ? threads : omp_get_num_procs());
#else
    (void)threads;
#endif
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t p = 0; p < n_pairs; p++) {
        const int64_t r = pair_read[p], h = pair_hap[p];
        const int64_t o = read_off[r];
        const int R = (int)(read_off[r + 1] - o);
        const int H = (int)(hap_off[h + 1] - hap_off[h]);
        out[p] = oracle_logless(hap_bases + hap_off[h], H, bases + o, quals + o, ins + o, del + o, gcp + o, R, 1);
    }
}

int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
