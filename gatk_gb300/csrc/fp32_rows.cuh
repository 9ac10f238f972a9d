// fp32_rows.cuh -- row coefficients and packed-float helpers shared by the FP32 wavefront kernels
// (fp32_bucket_kernel in kernels.cu, pd_bucket_kernel in pd_packed.cu).  Internal linkage: each translation unit
// that includes it gets its own copy.
#pragma once
#include <cuda_runtime.h>

#include <cstdint>

#include "ghmm_internal.h"

namespace ghmm {
namespace {

constexpr unsigned kFull = 0xffffffffu;
// log10(2^120) and log10(2^1020)
constexpr double kLog10Scale32 = 36.12359947967774;
constexpr double kLog10Scale64 = 307.0505955772608;

__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 zero2() { return make_float2(0.f, 0.f); }

__device__ __forceinline__ float2 shfl_up2(float2 v) {
    return make_float2(__shfl_up_sync(kFull, v.x, 1), __shfl_up_sync(kFull, v.y, 1));
}
__device__ __forceinline__ float2 shfl_down2(float2 v) {
    return make_float2(__shfl_down_sync(kFull, v.x, 1), __shfl_down_sync(kFull, v.y, 1));
}

__device__ __forceinline__ uint32_t base_code(uint8_t b) {
    switch (b) {
        case 'A': return 1u;
        case 'C': return 2u;
        case 'G': return 4u;
        case 'T': return 8u;
        case 'N': return 15u;
        default: return 0u;
    }
}

// Haplotype column codes carry a base index (A, C, G, T, N = 0..4); a read base matches index h when its
// mask shares a bit with kBaseMask[h] (N matches everything).
constexpr int kBases = 5;
__device__ __constant__ uint32_t kBaseMask[kBases] = {1u, 2u, 4u, 8u, 15u};

// Per-row coefficients of one read half (see header comment); dummy rows reproduce the row-0 boundary.
struct RowCoef {
    float pm, pe, b, c, e, dd;
    uint32_t code;
};

// Rows p = R and p = R + 1 below a read of R bases are its accumulator rows (kAccRows): row R+1 has prior 0
// and e = MI_R / MM_R, so I~(R+1, j) = M~(R, j) + (MI_R / MM_R) I~(R, j) = a_R (M + I)(R, j); row R+2 has
// prior 1, b = 1, c = 0, DD = 1, so M~(R+2, j) = I~(R+1, j-1) and D~(R+2, j) runs the sum over columns.  At a
// haplotype's last column H the likelihood numerator is D~(R+2, H) + M~(R+2, H) + I~(R+1, H) (sums through
// columns H-2, H-1 and H), and no per-step accumulation is left in the wavefront.
__device__ __forceinline__ RowCoef row_coef(const DevTables &T, const DevBatch &B, int64_t off, int R, int p) {
    RowCoef c;
    c.code = 0u;
    if (p < 0 || p > R + 1 || R == 0) {  // dummy row: holds the row-0 boundary
        c.pm = c.pe = 0.f;
        c.b = c.c = c.e = 0.f;
        c.dd = 1.f;
        return c;
    }
    if (p == R) {  // accumulator row R+1
        const uint8_t ins = B.ins[off + R - 1], del = B.dels[off + R - 1];
        c.pm = c.pe = 0.f;
        c.b = c.c = 0.f;
        c.e = __ldg(T.err_f + ins) / __ldg(T.m2m_f + ins * 128 + del);
        c.dd = 0.f;
        return c;
    }
    if (p == R + 1) {  // accumulator row R+2
        c.pm = c.pe = 1.f;
        c.b = 1.f;
        c.c = c.e = 0.f;
        c.dd = 1.f;
        return c;
    }
    const uint8_t base = B.bases[off + p], q = B.quals[off + p];
    const uint8_t ins = B.ins[off + p], del = B.dels[off + p], gcp = B.gcp[off + p];
    const float mm = __ldg(T.m2m_f + ins * 128 + del), mi = __ldg(T.err_f + ins), md = __ldg(T.err_f + del);
    const float im = __ldg(T.prob_f + gcp), ii = __ldg(T.err_f + gcp);
    float mm_p = 1.f, mi_p = 1.f, md_p = 1.f;
    if (p > 0) {
        const uint8_t ins_p = B.ins[off + p - 1], del_p = B.dels[off + p - 1];
        mm_p = __ldg(T.m2m_f + ins_p * 128 + del_p);
        mi_p = __ldg(T.err_f + ins_p);
        md_p = __ldg(T.err_f + del_p);
    }
    c.pm = __ldg(T.prob_f + q);
    c.pe = (base == 'N') ? c.pm : __ldg(T.err3_f + q);
    c.b = im * mi_p / (mm * mm_p);
    c.c = im * md_p / mm;
    c.e = (p > 0) ? ii * mi_p / (mi * mm_p) : 0.f;
    c.dd = ii;
    c.code = base_code(base);
    return c;
}

// log2(GHMM_FP32_RERUN_THRESHOLD) = log2(1e-28)
constexpr float kLog2Threshold = -93.01398f;

}  // namespace
}  // namespace ghmm
