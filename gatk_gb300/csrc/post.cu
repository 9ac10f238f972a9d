// post.cu -- the step after the likelihoods, fused on the device: per-read normalisation of the read-major
// likelihood blocks and the poorly-modelled-read filter, as PairHMMLikelihoodCalculationEngine.computeReadLikelihoods
// runs them after the PairHMM (src/main/java/org/broadinstitute/hellbender/tools/walkers/haplotypecaller/
// PairHMMLikelihoodCalculationEngine.java:200-201):
//   AlleleLikelihoods.normalizeLikelihoods (utils/genotyper/AlleleLikelihoods.java:416-458): per read, every
//     haplotype likelihood below best + cap is raised to best + cap, where best is searchBestAllele's (:505-540;
//     with symmetric = false the reference haplotype cannot be the best);
//   AlleleLikelihoods.filterPoorlyModeledEvidence (:1351-1376): a read whose best likelihood over all haplotypes
//     is below its threshold is dropped; the threshold is ReadLikelihoodCalculationEngine.log10MinTrueLikelihood
//     (ReadLikelihoodCalculationEngine.java:124-132) or, with dynamic disqualification, the smaller of that and
//     the DRAGEN-GATK read-quality threshold (:106-158).
// One thread per read; the read's block of n_haps doubles is rewritten in place and keep[read] is 0 or 1.
// The arithmetic is IEEE double with no contraction (explicit _rn intrinsics), so results equal Java's.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>

#include "ghmm_internal.h"

namespace ghmm {
namespace {

// (mean, variance) of the dynamic threshold per base quality 1..40 (ReadLikelihoodCalculationEngine.java:163-178)
__constant__ double kDynMean[40] = {
    5.996842844, 5.870018422, 5.401558531, 4.818940919, 4.218758304, 3.646319832, 3.122346753, 2.654731979,
    2.244479156, 1.88893867,  1.583645342, 1.3233807,   1.102785365, 0.916703025, 0.760361881, 0.629457387,
    0.520175654, 0.42918208,  0.353590663, 0.290923699, 0.23906788,  0.196230431, 0.160897421, 0.131795374,
    0.1078567,   0.088189063, 0.072048567, 0.058816518, 0.047979438, 0.039111985, 0.031862437, 0.025940415,
    0.021106532, 0.017163711, 0.013949904, 0.011332027, 0.009200898, 0.007467036, 0.006057179, 0.004911394};
__constant__ double kDynVar[40] = {
    0.196616587, 1.388545569, 5.641990128, 10.33176216, 14.25799688, 17.02880749, 18.64537883, 19.27521677,
    19.13584613, 18.43922003, 17.36842261, 16.07088712, 14.65952563, 13.21718577, 11.80207947, 10.45304833,
    9.194183767, 8.038657241, 6.991779595, 6.053379213, 5.219610436, 4.484302033, 3.839943445, 3.27839108,
    2.791361596, 2.370765375, 2.008921719, 1.698687797, 1.433525748, 1.207526336, 1.015402928, 0.852465956,
    0.714585285, 0.598145851, 0.500000349, 0.41742159,  0.348056286, 0.289881373, 0.241163527, 0.200422214};

__device__ double min_true_likelihood(int len, double rate, bool cap) {
    double e = ceil(__dmul_rn((double)len, rate));
    if (cap) e = fmin(2.0, e);
    return __dmul_rn(e, -4.0);
}

__global__ void postprocess_kernel(DevBatch B, int64_t n_reads, PostArgs P, uint8_t *keep) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += (int64_t)gridDim.x * blockDim.x) {
        const int g = B.read_region[r];
        const int nh = (int)(B.region_hap_off[g + 1] - B.region_hap_off[g]);
        double *row = B.out + B.out_off[g] + (r - B.region_read_off[g]) * (int64_t)nh;
        const int ref = P.reference_hap ? P.reference_hap[g] : -1;
        if (P.normalize && nh > 1) {
            // searchBestAllele
            double best = -INFINITY;
            if (!(nh == 1 && ref == 0 && !P.symmetric)) {
                const int b0 = (P.symmetric || ref != 0) ? 0 : 1;
                best = row[b0];
                for (int a = b0 + 1; a < nh; ++a) {
                    if (!P.symmetric && a == ref) continue;
                    if (row[a] > best) best = row[a];
                }
            }
            const double worst = __dadd_rn(best, P.cap);
            for (int a = 0; a < nh; ++a)
                if (row[a] < worst) row[a] = worst;
        }
        double mx = -INFINITY;
        for (int a = 0; a < nh; ++a)
            if (row[a] > mx) mx = row[a];
        const int64_t q0 = B.read_off[r];
        const int len = (int)(B.read_off[r + 1] - q0);
        double thr;
        if (P.dynamic) {
            double sm = 0.0, sv = 0.0;
            for (int i = 0; i < len; ++i) {
                const int bq = B.quals[q0 + i];
                const int e = bq <= 1 ? 0 : min(40, bq) - 1;
                sm = __dadd_rn(sm, kDynMean[e]);
                sv = __dadd_rn(sv, kDynVar[e]);
            }
            const double d = __dmul_rn(__dadd_rn(sm, __dmul_rn(P.scale, sqrt(sv))), -0.1);
            const double m = min_true_likelihood(len, P.rate, false);
            thr = d < m ? d : m;
        } else {
            thr = min_true_likelihood(len, P.rate, true);
        }
        keep[r] = (mx < thr) ? 0 : 1;
    }
}

}  // namespace

int launch_postprocess(const DevBatch &b, int64_t n_reads, const PostArgs &p, uint8_t *keep, int sm_count,
                       cudaStream_t s) {
    if (n_reads <= 0) return 0;
    const int block = 256;
    const int64_t want = (n_reads + block - 1) / block;
    const int grid = (int)(want < (int64_t)sm_count * 8 ? want : (int64_t)sm_count * 8);
    postprocess_kernel<<<grid, block, 0, s>>>(b, n_reads, p, keep);
    return (int)cudaGetLastError();
}

}  // namespace ghmm
