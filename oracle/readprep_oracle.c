/* readprep_oracle.c -- CPU restatement of the read preparation before the PairHMM, in C with OpenMP over reads.
 *
 * TEST INFRASTRUCTURE ONLY: the C twin of oracle/readprep.py for large samples (bench.py --prep's timed CPU baseline
 * and its parity check) and the tests.  The product never links it.
 *
 * Follows (paths inside the GATK repository):
 *   PairHMMLikelihoodCalculationEngine.modifyReadQualities / capMinimumReadQualities / setToFixedValueIfTooLow
 *       src/main/java/org/broadinstitute/hellbender/tools/walkers/haplotypecaller/
 *       PairHMMLikelihoodCalculationEngine.java:283-322
 *   PCR indel error model: initializePCRErrorModel, getErrorModelAdjustedQual, applyPCRErrorModel      :331-371
 *   ReadLikelihoodCalculationEngine.findTandemRepeatUnits (unit lengths up to 8, repeat lengths capped at 20)
 *       ReadLikelihoodCalculationEngine.java:25-26,193-253
 *   GATKVariantContextUtils.findNumberOfRepetitions   utils/variant/GATKVariantContextUtils.java:949-1011
 *   DragstrPairHMMInputScoreImputator.impute          tools/walkers/haplotypecaller/
 *       DragstrPairHMMInputScoreImputator.java:22-31,54-88
 *   DragstrReadSTRAnalyzer (most repeated period, ties to the shorter one)   utils/pairhmm/DragstrReadSTRAnalyzer.java
 *       :110-139, in the position-by-position definition of DragstrReadSTRAnalyzerTest.java:131-168
 *   DragstrParams.lookup                               utils/dragstr/DragstrParams.java:194-220
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define RP_MAX_UNIT 8
#define RP_MAX_REPEAT 20
#define RP_MIN_USABLE_Q 6
#define RP_DEFAULT_INDEL_Q 45
#define RP_PI 3.141592653589793

/* copies of unit[0, L) that test[0, n) starts with (leading) or ends with (trailing) */
static int repetitions(const uint8_t *unit, int L, const uint8_t *test, int n, int leading) {
    if (n == 0) return 0;
    int count = 0;
    if (leading) {
        for (int s = 0; s + L <= n; s += L) {
            if (memcmp(test + s, unit, (size_t)L) != 0) return count;
            count++;
        }
    } else {
        for (int s = n - L; s >= 0; s -= L) {
            if (memcmp(test + s, unit, (size_t)L) != 0) return count;
            count++;
        }
    }
    return count;
}

/* findTandemRepeatUnits(bases, offset).getRight(), capped at RP_MAX_REPEAT */
static int tandem_repeat_length(const uint8_t *b, int n, int offset) {
    int max_bw = 0, bw_start = offset, bw_len = 1;
    for (int L = 1; L <= RP_MAX_UNIT; L++) {
        if (offset + 1 - L < 0) break;
        max_bw = repetitions(b + offset - L + 1, L, b, offset + 1, 0);
        if (max_bw > 1) {
            bw_start = offset - L + 1;
            bw_len = L;
            break;
        }
    }
    int max_rl = max_bw;
    if (offset < n - 1) {
        int fw_len = 1, max_fw = 0;
        for (int L = 1; L <= RP_MAX_UNIT; L++) {
            if (offset + L + 1 > n) break;
            max_fw = repetitions(b + offset + 1, L, b + offset + 1, n - offset - 1, 1);
            if (max_fw > 1) {
                fw_len = L;
                break;
            }
        }
        const uint8_t *fw = b + offset + 1;
        if (fw_len == bw_len && memcmp(fw, b + bw_start, (size_t)fw_len) == 0)
            max_rl = max_bw + max_fw;
        else
            max_rl = max_fw + repetitions(fw, fw_len, b, offset + 1, 0);
    }
    return max_rl < RP_MAX_REPEAT ? max_rl : RP_MAX_REPEAT;
}

/* MathUtils.fastRound */
static int fast_round(double d) { return d > 0.0 ? (int)(d + 0.5) : (int)(d - 0.5); }

/* Math.round(double), half up */
static long long java_round(double x) {
    double r = floor(x);
    if (x - r >= 0.5) r += 1.0;
    return (long long)r;
}

static int as_java_byte(int v) { return v > 127 ? v - 256 : v; }

/* repeat count of `period` at `pos`: the longest tandem run, in units, of a period-mer containing pos or starting
 * right after it; a unit starting at 0 counts one fewer (not below 1) for positions before period - 1 */
static int str_repeats(const uint8_t *s, int n, int pos, int p) {
    if (p > n) return 0;
    int best = 0;
    for (int start = pos - p + 1 > 0 ? pos - p + 1 : 0; start <= pos + 1 && start + p <= n; start++) {
        const uint8_t *unit = s + start;
        int count = 1;
        for (int off = start + p; off + p <= n && memcmp(s + off, unit, (size_t)p) == 0; off += p) count++;
        for (int off = start - p; off >= 0 && memcmp(s + off, unit, (size_t)p) == 0; off -= p) count++;
        if (pos < p - 1 && start == 0) count = count - 1 > 1 ? count - 1 : 1;
        if (count > best) best = count;
    }
    return best;
}

/* DragstrPairHMMInputScoreImputator.impute: GOP (insertion = deletion) and GCP of one read */
static void dragstr_impute(const uint8_t *b, int n, const double *gop_t, const double *gcp_t, int maxp, int maxr,
                           uint8_t *gop, uint8_t *gcp) {
    if (n == 0) return;
    for (int i = 0; i < n - 1; i++) {
        int best_p = 1, best_r = str_repeats(b, n, i, 1);
        for (int p = 2; p <= maxp; p++) {
            const int r = str_repeats(b, n, i, p);
            if (r > best_r) best_p = p, best_r = r;
        }
        const int pi = best_p < maxp ? best_p - 1 : maxp - 1, ri = best_r < maxr ? best_r - 1 : maxr - 1;
        const double g = gop_t[pi * maxr + ri], c = gcp_t[pi * maxr + ri];
        gop[i] = (uint8_t)(java_round(g < 40.0 ? g : 40.0) & 0xFF);
        gcp[i] = (uint8_t)(java_round(c) & 0xFF);
    }
    gop[n - 1] = 45;
    gcp[n - 1] = 10;
}

/* The four prepared planes (base qualities, insertion GOP, deletion GOP, GCP) of n_reads reads laid back to back at
 * read_off.  ins / dels may be NULL (45 everywhere, ReadUtils' default); gop_t / gcp_t non-NULL select the DRAGstr
 * imputation ([max_period][max_repeats] tables) instead of the PCR model and the constant gcp.  threads <= 0: all
 * processors.  Returns 0. */
int rp_prepare_reads(int64_t n_reads, const int64_t *read_off, const uint8_t *bases, const uint8_t *quals,
                     const uint8_t *ins, const uint8_t *dels, const int32_t *mapq, int threshold, int cap_to_mapq,
                     double rate_factor, int gcp, const double *gop_t, const double *gcp_t, int max_period,
                     int max_repeats, uint8_t *out_q, uint8_t *out_i, uint8_t *out_d, uint8_t *out_g, int threads) {
    int cache[RP_MAX_REPEAT + 1];
    for (int rl = 0; rl <= RP_MAX_REPEAT; rl++) {
        const int q = rate_factor != 0.0 ? fast_round(40.0 - exp((double)rl / (rate_factor * RP_PI)) + 1.0) : 40;
        cache[rl] = q > 10 ? q : 10;
    }
    const int dragstr = gop_t != NULL && gcp_t != NULL;
#ifdef _OPENMP
    if (threads <= 0) threads = omp_get_num_procs();
#pragma omp parallel for schedule(dynamic, 256) num_threads(threads)
#endif
    for (int64_t r = 0; r < n_reads; r++) {
        const int64_t o = read_off[r];
        const int n = (int)(read_off[r + 1] - o);
        const uint8_t *b = bases + o;
        for (int i = 0; i < n; i++) {
            int q = quals[o + i];
            if (cap_to_mapq) q = (q < mapq[r] ? q : mapq[r]) & 0xFF;
            out_q[o + i] = (uint8_t)(as_java_byte(q) < threshold ? RP_MIN_USABLE_Q : q);
        }
        if (dragstr) {
            dragstr_impute(b, n, gop_t, gcp_t, max_period, max_repeats, out_i + o, out_g + o);
            memcpy(out_d + o, out_i + o, (size_t)n);
            continue;
        }
        for (int i = 0; i < n; i++) {
            out_i[o + i] = ins ? ins[o + i] : RP_DEFAULT_INDEL_Q;
            out_d[o + i] = dels ? dels[o + i] : RP_DEFAULT_INDEL_Q;
            out_g[o + i] = (uint8_t)gcp;
        }
        if (rate_factor != 0.0) {  /* applyPCRErrorModel: unsigned minimum with the model's quality */
            for (int i = 1; i < n; i++) {
                const int cap = cache[tandem_repeat_length(b, n, i - 1)];
                if (out_i[o + i - 1] > cap) out_i[o + i - 1] = (uint8_t)cap;
                if (out_d[o + i - 1] > cap) out_d[o + i - 1] = (uint8_t)cap;
            }
        }
        for (int i = 0; i < n; i++) {  /* capMinimumReadQualities' floors, as Java's signed bytes */
            if (as_java_byte(out_i[o + i]) < RP_MIN_USABLE_Q) out_i[o + i] = RP_MIN_USABLE_Q;
            if (as_java_byte(out_d[o + i]) < RP_MIN_USABLE_Q) out_d[o + i] = RP_MIN_USABLE_Q;
        }
    }
    return 0;
}
