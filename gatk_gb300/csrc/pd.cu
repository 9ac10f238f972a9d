// pd.cu -- the partially-determined-haplotype PairHMM (PD-HMM) forward on the GPU.
//
// The recurrence is LoglessPDPairHMM's (src/main/java/org/broadinstitute/hellbender/utils/pairhmm/
// LoglessPDPairHMM.java:35-150): LoglessPairHMM's M/I/D plus three branch matrices bM/bI/bD that carry the state
// from before an undetermined deletion.  Along a row every column is processed in one of three states, set by the
// PD flags of the previous column (DEL_START enters INSIDE_DEL, DEL_END enters AFTER_DEL, AFTER_DEL lasts one
// column):
//    NORMAL:     bX(i,j) = X(i,j-1)
//    INSIDE_DEL: bX(i,j) = bX(i,j-1)
//    AFTER_DEL:  bX(i,j) = max(bX(i,j-1), X(i,j-1)), and M and D read max(bX, X) of their diagonal / left inputs
// and at a DEL_END column I reads max(bX, X) of the row above.  The state carries from the end of one row to the
// start of the next, so row 1 and rows >= 2 can see different states at the first columns; the host computes both
// sequences per haplotype column (pd_attach in runtime.cpp) and the kernel takes row 1's for the read's first row.
// The prior also matches a read base against an undetermined SNP's alternative (isBasePDMatching, :196-210).
//
// Kernel: one (read, haplotype) pair per warp, K rows per lane (K = 1..4, per read the strip height that wastes the
// fewest padding rows), the anti-diagonal wavefront of the FP64 kernels in kernels.cu with six values per row,
// strips of 32*K rows through per-warp scratch (six values per column).  Steps where no lane of the warp is at an
// AFTER_DEL or DEL_END column (nearly all) take a path without max(); the rest take the general one.  Two precisions
// of the same code:
//   double: the reference's scale 2^1020 and FP64 arithmetic (GHMM_MODE_PD, and the reruns below);
//   float:  scale 2^120, FP32 arithmetic (64 times the FP64 rate on this part); a sum below
//           GHMM_FP32_RERUN_THRESHOLD at that scale, or not finite, queues the pair for the FP64 kernel, as the
//           regular FP32 pass does (GHMM_MODE_PD_FP32).
#include <cuda_runtime.h>

#include <cfloat>
#include <cmath>
#include <cstdint>
#include <type_traits>

#include "ghmm_internal.h"

namespace ghmm {
namespace {

constexpr unsigned kFull = 0xffffffffu;
constexpr double kLog10Scale = 307.0505955772608;    // log10(2^1020)
constexpr double kLog10Scale32 = 36.12359947967774;  // log10(2^120)
constexpr float kLog2Threshold = -93.01398f;         // log2(GHMM_FP32_RERUN_THRESHOLD)
constexpr int kPdBlock = 128;

__device__ __forceinline__ double vfma(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ float vfma(float a, float b, float c) { return fmaf(a, b, c); }
__device__ __forceinline__ double vmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ float vmax(float a, float b) { return fmaxf(a, b); }

// The transition and prior tables in the kernel's precision
template <typename V>
struct PdTab;
template <>
struct PdTab<double> {
    const double *prob, *err3, *m2m, *err;
    __device__ explicit PdTab(const DevTables &T) : prob(T.prob_d), err3(T.err3_d), m2m(T.m2m_d), err(T.err_d) {}
};
template <>
struct PdTab<float> {
    const float *prob, *err3, *m2m, *err;
    __device__ explicit PdTab(const DevTables &T) : prob(T.prob_f), err3(T.err3_f), m2m(T.m2m_f), err(T.err_f) {}
};

__device__ __forceinline__ uint32_t pd_base_bit(uint32_t x) {
    switch (x) {
        case 'A': case 'a': return 8u;
        case 'C': case 'c': return 16u;
        case 'G': case 'g': return 32u;
        case 'T': case 't': return 64u;
        default: return 0u;
    }
}

// Pairs [begin, begin + count) of the batch's pair list (count_dev: the count in device memory instead), all of
// whose reads take K rows per lane: the host picks, per read, the strip height 32 K (K = 1..4) that wastes the fewest
// padding rows (K = 1..4 in FP64, 1..8 in FP32); FP64 reruns all take K = 4.
template <typename V, int K>
__global__ void __launch_bounds__(kPdBlock, (sizeof(V) == 4 && K <= 4) ? 4 : 3) pd_kernel(DevTables TT, DevBatch B, PdPlanes P, int begin, int count,
                                                         int cursor, const int32_t *count_dev) {
    constexpr bool F32 = sizeof(V) == 4;
    constexpr int S = 32 * K;
    const PdTab<V> T(TT);
    const int lane = threadIdx.x & 31;
    const int64_t warp_global = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    V *scratch = reinterpret_cast<V *>(B.scratch64) + warp_global * B.scratch64_cols * 6;
    if (count_dev) count = min(*count_dev, (int)B.rerun_capacity);
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&B.counters[cursor], 1);
        t = __shfl_sync(kFull, t, 0);
        if (t >= count) break;
        const PairRef pr = B.rerun[begin + t];
        const int read = pr.read, hap = pr.hap;
        const int64_t roff = B.read_off[read];
        const int R = (int)(B.read_off[read + 1] - roff);
        const int64_t hoff = B.hap_off[hap];
        const int H = (int)(B.hap_off[hap + 1] - hoff);
        const int region = B.read_region[read];
        const int64_t nh = B.region_hap_off[region + 1] - B.region_hap_off[region];
        const int64_t out_index = B.out_off[region] + (int64_t)(read - B.region_read_off[region]) * nh +
                                  (hap - B.region_hap_off[region]);
        if (R == 0 || H == 0) {
            if (lane == 0) B.out[out_index] = -INFINITY;
            continue;
        }
        if (H > B.scratch64_cols && R > S) {
            if (lane == 0) atomicExch(&B.counters[3], 2);
            continue;
        }
        const V init = F32 ? (V)B.hap_init_f[hap] : (V)B.hap_init_d[hap];
        const int nstrips = (R + S - 1) / S;
        const int pad = nstrips * S - R;
        const uint8_t *hb = B.hap_bases + hoff;
        const uint8_t *hf = P.flags + hoff;
        const uint8_t *hs = P.states + hoff;
        V acc = 0;
        for (int strip = 0; strip < nstrips; ++strip) {
            // tii doubles as DD (equal for read rows); a dummy row has tii = 1 so its D holds the row-0 value and its
            // I stays at the (zero) value above it
            // the prior is folded into M's coefficients: (prior x MM, prior x IM) for a match and a mismatch, so a
            // cell's M costs one multiply and two fused multiply-adds (on this part a DMUL or DADD issues at about
            // 0.85 of the DFMA rate)
            V mMM[K], mIM[K], eMM[K], eIM[K], tmi[K], tii[K], tmd[K];
            uint32_t rbase[K], rbit[K];
            bool first[K], dummy[K], rN[K];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int p = strip * S + lane * K + k - pad;
                dummy[k] = p < 0;
                first[k] = p == 0;
                if (p < 0) {
                    mMM[k] = mIM[k] = eMM[k] = eIM[k] = 0;
                    tmi[k] = tmd[k] = 0;
                    tii[k] = 1;
                    rbase[k] = 0x100u;
                    rN[k] = false;
                    rbit[k] = 0u;
                } else {
                    const uint8_t base = B.bases[roff + p], q = B.quals[roff + p];
                    const uint8_t ins = B.ins[roff + p], del = B.dels[roff + p], gcp = B.gcp[roff + p];
                    const V pm = __ldg(T.prob + q), pe = __ldg(T.err3 + q);
                    const V mm = __ldg(T.m2m + ins * 128 + del), im = __ldg(T.prob + gcp);
                    mMM[k] = pm * mm;
                    mIM[k] = pm * im;
                    eMM[k] = pe * mm;
                    eIM[k] = pe * im;
                    tmi[k] = __ldg(T.err + ins);
                    tii[k] = __ldg(T.err + gcp);
                    tmd[k] = __ldg(T.err + del);
                    rbase[k] = base;
                    rN[k] = base == 'N';
                    rbit[k] = pd_base_bit(base);
                }
            }
            V Mp[K], Ip[K], Dp[K], bM[K], bI[K], bD[K];
            auto reset = [&]() {
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    Mp[k] = Ip[k] = 0;
                    Dp[k] = dummy[k] ? init : (V)0;
                    bM[k] = bI[k] = bD[k] = 0;
                }
            };
            reset();
            V gM = 0, gI = 0, gbM = 0, gbI = 0, gbD = 0;
            const bool above_dummy = (strip == 0) && (lane * K - 1 < pad);
            V gD = above_dummy ? init : (V)0;
            const bool last_strip = strip == nstrips - 1;
            V nx[6] = {0, 0, 0, 0, 0, 0};
            if (strip > 0 && lane == 0)
#pragma unroll
                for (int v = 0; v < 6; ++v) nx[v] = scratch[v];
            const int nsteps = H + 31;
            // one wavefront step; CHK steps handle lanes outside the haplotype's columns and the column-0 reset, which
            // fall in the first 32 and the last 31 steps only
            auto step = [&](const int s, auto chk_tag) {
                constexpr bool CHK = decltype(chk_tag)::value;
                const int c = s - lane;
                const bool valid = !CHK || (c >= 0 && c < H);
                uint32_t y = 0x200u, f = 0u, st = 0u;
                if (valid) {
                    y = __ldg(hb + c);
                    f = __ldg(hf + c);
                    st = __ldg(hs + c);
                }
                if (CHK && c == 0) {  // column-0 boundary: M = I = D = 0 (row 0: D = scale / H), branches 0
                    reset();
                    gM = gI = gbM = gbI = gbD = 0;
                    gD = above_dummy ? init : (V)0;
                }
                V u[6];
                u[0] = __shfl_up_sync(kFull, Mp[K - 1], 1);
                u[1] = __shfl_up_sync(kFull, Ip[K - 1], 1);
                u[2] = __shfl_up_sync(kFull, Dp[K - 1], 1);
                u[3] = __shfl_up_sync(kFull, bM[K - 1], 1);
                u[4] = __shfl_up_sync(kFull, bI[K - 1], 1);
                u[5] = __shfl_up_sync(kFull, bD[K - 1], 1);
                if (lane == 0) {
                    if (strip == 0) {
                        u[0] = u[1] = u[3] = u[4] = u[5] = 0;
                        u[2] = init;
                    } else {
#pragma unroll
                        for (int v = 0; v < 6; ++v) u[v] = nx[v];
                        if (c + 1 < H)
#pragma unroll
                            for (int v = 0; v < 6; ++v) nx[v] = scratch[6 * (c + 1) + v];
                    }
                }
                const uint32_t st1 = st & 3u, st2 = (st >> 2) & 3u;
                const bool del_end = (st & 16u) != 0;
                const bool yn = (y == 'N');
                // the general path only when a lane of this warp sits at an AFTER_DEL or DEL_END column
                const bool special = __any_sync(kFull, valid && (st1 == 2u || st2 == 2u || del_end));
                // pass 1 (bottom-up, the row above still holds the previous column): branches, M, D.  PLAIN: every
                // lane's column is NORMAL for all its rows (no deletion state) and is neither an undetermined SNP nor
                // an N (the common case), so the branch states just take the previous column's values and a read
                // base matches the column exactly when it equals it or is N
                auto pass1 = [&](auto plain_tag) {
                    constexpr bool PLAIN = decltype(plain_tag)::value;
#pragma unroll
                    for (int k = K - 1; k >= 0; --k) {
                        const V dM = k ? Mp[k - 1] : gM, dI = k ? Ip[k - 1] : gI, dD = k ? Dp[k - 1] : gD;
                        const bool match = PLAIN ? (rbase[k] == y || rN[k])
                                                 : (rbase[k] == y || rN[k] || yn || ((f & 1u) && (f & rbit[k])));
                        const V cMM = match ? mMM[k] : eMM[k], cIM = match ? mIM[k] : eIM[k];
                        V Mn, Dn, nbM, nbI, nbD;
                        if (PLAIN) {
                            nbM = Mp[k];
                            nbI = Ip[k];
                            nbD = Dp[k];
                            Mn = vfma(dM, cMM, vfma(dI, cIM, dD * cIM));
                            Dn = vfma(Dp[k], tii[k], Mp[k] * tmd[k]);
                        } else {
                            const uint32_t sk = first[k] ? st1 : st2;
                            if (special && sk == 2u) {
                                const V dbM = k ? bM[k - 1] : gbM, dbI = k ? bI[k - 1] : gbI;
                                const V dbD = k ? bD[k - 1] : gbD;
                                nbM = vmax(bM[k], Mp[k]);
                                nbI = vmax(bI[k], Ip[k]);
                                nbD = vmax(bD[k], Dp[k]);
                                Mn = vfma(vmax(dbM, dM), cMM, vfma(vmax(dbI, dI), cIM, vmax(dbD, dD) * cIM));
                                Dn = vfma(vmax(bD[k], Dp[k]), tii[k], vmax(bM[k], Mp[k]) * tmd[k]);
                            } else {
                                const bool inside = sk == 1u;
                                nbM = inside ? bM[k] : Mp[k];
                                nbI = inside ? bI[k] : Ip[k];
                                nbD = inside ? bD[k] : Dp[k];
                                Mn = vfma(dM, cMM, vfma(dI, cIM, dD * cIM));
                                Dn = vfma(Dp[k], tii[k], Mp[k] * tmd[k]);
                            }
                        }
                        if (CHK && !valid) Mn = Dn = 0, nbM = nbI = nbD = 0;
                        Mp[k] = Mn;
                        Dp[k] = Dn;
                        bM[k] = nbM;
                        bI[k] = nbI;
                        bD[k] = nbD;
                    }
                };
                if constexpr (!CHK && F32) {  // (the FP64 kernels keep one form: registers, not issue, bind them)
                    if (!__any_sync(kFull, st != 0u || (f & 1u) || yn))
                        pass1(std::true_type{});
                    else
                        pass1(std::false_type{});
                } else {
                    pass1(std::false_type{});
                }
                // pass 2 (top-down): I from the row above at this column
                V aM = u[0], aI = u[1], abM = u[3], abI = u[4];
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    V In;
                    if (special && del_end)
                        In = vfma(vmax(abI, aI), tii[k], vmax(abM, aM) * tmi[k]);
                    else
                        In = vfma(aI, tii[k], aM * tmi[k]);
                    if (CHK && !valid) In = 0;
                    Ip[k] = In;
                    aM = Mp[k];
                    aI = In;
                    abM = bM[k];
                    abI = bI[k];
                }
                gM = u[0];
                gI = u[1];
                gD = u[2];
                gbM = u[3];
                gbI = u[4];
                gbD = u[5];
                if (valid && lane == 31) {
                    if (last_strip) {
                        acc += Mp[K - 1] + Ip[K - 1];
                    } else {
                        V *d = scratch + 6 * c;
                        d[0] = Mp[K - 1];
                        d[1] = Ip[K - 1];
                        d[2] = Dp[K - 1];
                        d[3] = bM[K - 1];
                        d[4] = bI[K - 1];
                        d[5] = bD[K - 1];
                    }
                }
            };
            int s = 0;
            for (; s < nsteps && s < 32; ++s) step(s, std::true_type{});
#pragma unroll 2
            for (; s < H; ++s) step(s, std::false_type{});  // every lane at a column in 1 .. H - 1 (2.6 % faster unrolled)
            for (; s < nsteps; ++s) step(s, std::true_type{});
            __syncwarp();
        }
        if (lane == 31) {
            if (!F32) {
                B.out[out_index] = log10((double)acc) - kLog10Scale;
            } else if (acc > 0.f && acc <= FLT_MAX && log2f((float)acc) >= kLog2Threshold) {
                B.out[out_index] = log10((double)acc) - kLog10Scale32;
            } else {  // underflow at 2^120 (or not finite): the FP64 kernel recomputes the pair
                const int idx = atomicAdd(&B.counters[kCounterPdRerun], 1);
                if ((int64_t)idx < B.rerun_capacity)
                    B.rerun[B.rerun_capacity + idx] = pr;
                else
                    atomicExch(&B.counters[3], 1);
            }
        }
    }
}

}  // namespace

int pd_kernel_occupancy(int *blocks_per_sm) {
    // the FP64 variants run on one grid and scratch: the smallest occupancy of them (FP32 variants: launch_pd)
    int best = 1 << 30;
    const void *fns[] = {(const void *)pd_kernel<double, 1>, (const void *)pd_kernel<double, 2>,
                         (const void *)pd_kernel<double, 3>, (const void *)pd_kernel<double, 4>};
    for (const void *fn : fns) {
        int n = 0;
        const cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kPdBlock, 0);
        if (e != cudaSuccess) return (int)e;
        best = n < best ? n : best;
    }
    *blocks_per_sm = best;
    return 0;
}

int launch_pd(const DevTables &t, const DevBatch &b, const PdPlanes &p, int k, bool fp32, int begin, int count,
              int cursor, const int32_t *count_dev, int grid, cudaStream_t s) {
    // grid is the FP64 kernels' (the strip scratch is sized for it, six doubles per column and warp); an FP32
    // variant fits as many more resident blocks as its registers allow, up to twice that grid in the same scratch
    auto f32_grid = [&](const void *fn) {
        int n = 0, dev = 0, sms = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kPdBlock, 0) != cudaSuccess || n <= 0) return grid;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        const int want = n * sms;
        return want < 2 * grid ? (want > grid ? want : grid) : 2 * grid;
    };
#define GHMM_PD_CASE(KK)                                                                                      \
    case KK:                                                                                                  \
        if (fp32)                                                                                             \
            pd_kernel<float, KK><<<f32_grid((const void *)pd_kernel<float, KK>), kPdBlock, 0, s>>>(          \
                t, b, p, begin, count, cursor, count_dev);                                                    \
        else                                                                                                  \
            pd_kernel<double, KK><<<grid, kPdBlock, 0, s>>>(t, b, p, begin, count, cursor, count_dev);        \
        break;
#define GHMM_PD_CASE32(KK)                                                                                    \
    case KK:                                                                                                  \
        if (!fp32) return (int)cudaErrorInvalidValue;                                                         \
        pd_kernel<float, KK><<<f32_grid((const void *)pd_kernel<float, KK>), kPdBlock, 0, s>>>(              \
            t, b, p, begin, count, cursor, count_dev);                                                        \
        break;
    switch (k) {
        GHMM_PD_CASE(1)
        GHMM_PD_CASE(2)
        GHMM_PD_CASE(3)
        GHMM_PD_CASE(4)
        GHMM_PD_CASE32(5)
        GHMM_PD_CASE32(6)
        GHMM_PD_CASE32(7)
        GHMM_PD_CASE32(8)
        default: return (int)cudaErrorInvalidValue;
    }
#undef GHMM_PD_CASE
#undef GHMM_PD_CASE32
    return (int)cudaGetLastError();
}

}  // namespace ghmm
