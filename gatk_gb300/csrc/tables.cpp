// tables.cpp -- host construction of the Phred lookup tables the kernels read.
//
// Restates, for the product, the reference's tables:
//   QualityUtils.qualToErrorProbCache   QualityUtils.java:48-57 (10^(-q/10), q = 0..254)
//   QualityUtils.qualToProb(byte)       QualityUtils.java:83-85 (1 - error)
//   MathUtils.JacobianLogTable          MathUtils.java:406-430 (step 1e-4, tolerance 8)
//   MathUtils.approximateLog10SumLog10  MathUtils.java:467-480
//   PairHMMModel.matchToMatchProb       PairHMMModel.java:86-94,373-388
// evaluated in IEEE double with no fused multiply-add (the file is compiled with -ffp-contract=off), the
// same operations Java performs, so the FP64 kernels see the reference's exact transition values.
#include <cmath>
#include <vector>

#include "tables.h"

namespace ghmm {

namespace {

constexpr double kJacMaxTolerance = 8.0;
constexpr double kJacStep = 0.0001;

int fast_round(double d) { return (d > 0.0) ? (int)(d + 0.5) : (int)(d - 0.5); }

struct Jacobian {
    std::vector<double> cache;
    double inv_step;
    Jacobian() {
        inv_step = 1.0 / kJacStep;
        const int n = (int)(kJacMaxTolerance / kJacStep) + 1;
        cache.resize((size_t)n);
        for (int k = 0; k < n; k++) cache[(size_t)k] = std::log10(1.0 + std::pow(10.0, -((double)k) * kJacStep));
    }
    double approx_sum(double a, double b) const {
        if (a > b) return approx_sum(b, a);
        if (a == -INFINITY) return b;
        const double diff = b - a;
        return b + (diff < kJacMaxTolerance ? cache[(size_t)fast_round(diff * inv_step)] : 0.0);
    }
};

}  // namespace

void build_host_tables(HostTables &t) {
    for (int q = 0; q < 256; q++) {
        if (q <= kMaxQual) {
            t.err[q] = std::pow(10.0, ((double)q) / -10.0);
            t.prob[q] = 1.0 - t.err[q];
            t.err3[q] = t.err[q] / 3.0;
        } else {  // byte 255 is rejected by input validation; keep the slot finite
            t.err[q] = t.err[kMaxQual];
            t.prob[q] = t.prob[kMaxQual];
            t.err3[q] = t.err3[kMaxQual];
        }
    }
    const Jacobian jac;
    const double inv_ln10 = 1.0 / std::log(10.0);
    // matchToMatchProb[(max*(max+1))/2 + min]; expanded here to a full 128x128 (ins, del) table since
    // gap-open penalties are validated to 0..127 (Java signed bytes >= 0, PairHMMModel.java:109-111).
    for (int i = 0; i < 128; i++)
        for (int j = 0; j < 128; j++) {
            const int mx = i > j ? i : j, mn = i > j ? j : i;
            const double log10_sum = jac.approx_sum(-0.1 * mx, -0.1 * mn);
            double p = std::pow(10.0, log10_sum);
            if (p > 1.0) p = 1.0;
            const double l10 = std::log1p(-p) * inv_ln10;
            t.m2m[i * 128 + j] = std::pow(10.0, l10);
        }
    for (int q = 0; q < 256; q++) {
        t.err_f[q] = (float)t.err[q];
        t.prob_f[q] = (float)t.prob[q];
        t.err3_f[q] = (float)t.err3[q];
    }
    for (int k = 0; k < 128 * 128; k++) {
        t.m2m_f[k] = (float)t.m2m[k];
        t.lm2m[k] = t.m2m_f[k] > 0.0f ? -std::log2((double)t.m2m_f[k]) : 0.0;  // MM = 0 reads never run in FP32
    }
}

}  // namespace ghmm
