// tables.h -- host-side Phred lookup tables (see tables.cpp).
#pragma once

namespace ghmm {

constexpr int kMaxQual = 254;  // QualityUtils.MAX_QUAL, QualityUtils.java:43

struct HostTables {
    double err[256], prob[256], err3[256];
    double m2m[128 * 128];
    float err_f[256], prob_f[256], err3_f[256];
    float m2m_f[128 * 128];
    double lm2m[128 * 128];  // -log2(m2m_f): the FP32 pass's per-row rescaling exponent (kernels.cu read_scale_kernel)
};

void build_host_tables(HostTables &t);

}  // namespace ghmm
