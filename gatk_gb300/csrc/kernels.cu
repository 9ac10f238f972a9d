// kernels.cu -- sm_103a kernels of the GB300 PairHMM.
//
// The recurrence is LoglessPairHMM's (src/main/java/org/broadinstitute/hellbender/utils/pairhmm/
// LoglessPairHMM.java:47-67): for matrix row i (read position i-1) and column j (haplotype position j-1),
//   M(i,j) = prior(i,j) * (M(i-1,j-1)*MM_i + I(i-1,j-1)*IM_i + D(i-1,j-1)*IM_i)
//   I(i,j) = M(i-1,j)*MI_i + I(i-1,j)*II_i
//   D(i,j) = M(i,j-1)*MD_i + D(i,j-1)*DD_i
// with D(0,j) = scale/H, every other row-0 and column-0 entry 0, and
// log10 L = log10(sum_j M(R,j) + I(R,j)) - log10(scale).
//
// Three kernels:
//  * fp32_bucket_kernel<K, MULTI>: the batched FP32 forward.  One warp runs a read-pair task: two reads of
//    one region, packed into the .x/.y halves of float2 so every cell update is a packed FFMA2/FMUL2/FADD2,
//    against all (or a chunk of) the region's haplotypes streamed back to back.  Lane l owns K consecutive
//    rows; at step s it computes column c = s - 2l, receiving the row above from lane l-1 by __shfl_up_sync
//    (an anti-diagonal wavefront with a skew of two columns per lane, so that a value shuffled at the start of
//    a step is consumed one step later and the shuffle's latency stays off the per-step chain); lane l-1 hands
//    lane l two packed values per step, its row 0's I~ at a column and the inner sum b I~ + c D~ + M~ of its
//    row 0's M~ at the next column, computed with lane l's row-0 coefficients, instead of three raw states
//    (K >= 2).  Each read is followed by two accumulator rows that sum the last row over
//    the haplotype (row_coef), and padded at the top with "dummy" rows that reproduce the row-0 boundary, so
//    the accumulator rows always sit in lane 31's last two slots.  Reads longer than 32*K rows run
//    as several strips whose boundary row goes through per-warp global scratch.  Each row's states are
//    rescaled so a cell costs 5 FMA-pipe operations instead of 8: with a_0 = 1, a_i = a_{i-1} / MM_i,
//       M~ = a_i M,   I~ = (a_{i-1} / MI_i) I,   D~ = (a_i / MD_i) D,
//    the recurrence becomes
//       M~ = prior * fma(I~_diag, b_i, fma(D~_diag, c_i, M~_diag))
//       I~ = fma(I~_up, e_i, M~_up)
//       D~ = fma(D~_left, DD_i, M~_left)
//    with b_i = IM_i MI_{i-1} / (MM_i MM_{i-1}), c_i = IM_i MD_{i-1} / MM_i, e_i = II_i MI_{i-1} / (MI_i MM_{i-1})
//    (MM_0 = MI_0 = MD_0 = 1) and  M_R + I_R = (M~_R + I~_R MI_R / MM_R) / a_R.  Only ratios of adjacent rows'
//    coefficients appear; log2 a_R is summed per read once per upload (read_scale_kernel, in FP64 and in an order
//    fixed by the read, so a read's result is the same whatever task or batch it runs in).  Reads whose I~ could
//    outgrow FP32 (steeply rising insertion penalties) or whose MM is 0 are sent to FP64 by the host.
//    Scale 2^120; a sum below GHMM_FP32_RERUN_THRESHOLD (or not finite) queues the pair for FP64.
//  * fp64_queue_kernel<K, RESCALED>: the FP64 wavefront, one pair per warp, used for reruns and
//    double-precision mode: a rescaled tier (5 DP operations per cell) and an exact unscaled tier (scale
//    2^1020, LoglessPairHMM's magnitudes) for results near the bottom of the FP64 range.
//  * plain_fp64_kernel: the plain form, one pair per thread block sweeping anti-diagonals through shared
//    memory with a block barrier per diagonal, Java's operation order, one launch per region.
#include <cuda_runtime.h>
#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "../../include/ghmm.h"
#include "fp32_rows.cuh"
#include "ghmm_internal.h"

namespace ghmm {

namespace {

// t = a_R (M_R + I_R) summed over the haplotype (scaled by 2^120); the read's scale (s, n) from read_scale_kernel
// splits log2 a_R = n - log2 s into an integer n and a factor s in [2^-1/2, 2^1/2].  Accepted sums are stored raw
// as the float pair (t s, n) in the output slot; finalize_fp32_kernel turns them into log10 in FP64 with every lane
// busy, rather than one lane per warp running the FP64 log10 here on the 1/64-rate FP64 pipe.
__device__ __forceinline__ void emit_fp32(const DevBatch &B, float t, float2 scale, int read, int hap,
                                          int64_t out_index) {
    t *= scale.x;
    const float la = scale.y;
    const bool forced = B.force_rerun_every > 0 && out_index % B.force_rerun_every == 0;  // test hook
    if (t > 0.f && t <= FLT_MAX && log2f(t) - la >= kLog2Threshold && !forced) {
        reinterpret_cast<float2 *>(B.out)[out_index] = make_float2(t, la);
    } else {
        const int idx = atomicAdd(&B.counters[1], 1);
        if ((int64_t)idx < B.rerun_capacity) {
            B.rerun[idx].read = read;
            B.rerun[idx].hap = hap;
        } else {
            atomicExch(&B.counters[3], 1);
        }
    }
}

}  // namespace

// Blocks of 128 threads the FP32 kernel asks ptxas to fit per SM (register budget 65536 / (128 * n)).  K <= 5 fits
// four without spilling (126 registers at K = 5: 0.4 % faster than three); K = 6 and 7 at four spill a little and
// ran 1-2 % slower, K = 8 spills 600 bytes.
template <int K>
struct Fp32MinBlocks {
    static constexpr int value = K >= 6 ? 3 : 4;
};

// The bucket's task range and cursor live in device memory (B.bucket_info, B.counters), so the launch
// arguments do not depend on the batch and a captured CUDA graph can be replayed for every batch.
template <int K, bool MULTI>
__global__ void __launch_bounds__(128, Fp32MinBlocks<K>::value) fp32_bucket_kernel(DevTables T, DevBatch B) {
    constexpr int KEY = K | (MULTI ? 16 : 0);
    const int task_begin = B.bucket_info[KEY], task_count = B.bucket_info[kNumBucketKeys + KEY];
    const int counter_slot = kCounterBucketBase + KEY;
    constexpr int S = 32 * K;
    const int lane = threadIdx.x & 31;
    // Per-warp prior table in shared memory: prior[k/2][base][lane] holds rows k and k+1 as (read A, read B,
    // read A, read B), base index A,C,G,T,N = 0..4.  One 128-bit load per row pair and step replaces four
    // compares and four selects.
    constexpr int KP = (K + 1) / 2;  // row pairs
    extern __shared__ float4 prior_smem4[];
    float4 *prior_tbl4 = prior_smem4 + (size_t)(threadIdx.x >> 5) * (KP * kBases * 32) + lane;
    float2 *prior_tbl2 = reinterpret_cast<float2 *>(prior_tbl4);
    const int64_t warp_global = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    float2 *scratch = nullptr;
    if (MULTI) scratch = B.scratch32 + warp_global * B.scratch32_cols * 3;

    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&B.counters[counter_slot], 1);
        t = __shfl_sync(kFull, t, 0);
        if (t >= task_count) break;
        const F32Task task = B.tasks[task_begin + t];
        const int ra = task.read_a, rb = task.read_b;
        const int64_t off_a = B.read_off[ra];
        const int len_a = (int)(B.read_off[ra + 1] - off_a);
        int64_t off_b = 0;
        int len_b = 0;
        if (rb >= 0) {
            off_b = B.read_off[rb];
            len_b = (int)(B.read_off[rb + 1] - off_b);
        }
        const int region = task.region;
        const int64_t hap0 = B.region_hap_off[region];
        const int nh = (int)(B.region_hap_off[region + 1] - hap0);
        const int64_t rr0 = B.region_read_off[region];
        const int64_t out_a = B.out_off[region] + (int64_t)(ra - rr0) * nh - hap0;
        const int64_t out_b = B.out_off[region] + (int64_t)(rb - rr0) * nh - hap0;
        const int64_t col0 = B.hap_off[task.hap_begin];
        const int ncols = (int)(B.hap_off[task.hap_end] - col0);
        const uint8_t *stream = B.hap_code + col0;
        const int nstrips = MULTI ? task.nstrips : 1;

        for (int strip = 0; strip < nstrips; ++strip) {
            float2 cb[K], cc[K], ce[K], cdd[K];
            __syncwarp();  // the previous strip's steps have finished reading this warp's table
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int slot = strip * S + lane * K + k;
                const RowCoef a = row_coef(T, B, off_a, len_a, slot - task.pad_a);
                const RowCoef b = row_coef(T, B, off_b, rb >= 0 ? len_b : 0, slot - task.pad_b);
                cb[k] = make_float2(a.b, b.b);
                cc[k] = make_float2(a.c, b.c);
                ce[k] = make_float2(a.e, b.e);
                cdd[k] = make_float2(a.dd, b.dd);
#pragma unroll
                for (int h = 0; h < kBases; ++h) {
                    const uint32_t hm = kBaseMask[h];
                    prior_tbl2[((k / 2) * kBases + h) * 64 + (k & 1)] =
                        make_float2((a.code & hm) ? a.pm : a.pe, (b.code & hm) ? b.pm : b.pe);
                }
            }
            // row-0 coefficients of the lane below (lane 31: of the next strip's first row), with which this lane
            // hands it its row 0's I~ and M~ inner sum instead of three raw states
            float2 b0n = shfl_down2(cb[0]), c0n = shfl_down2(cc[0]), e0n = shfl_down2(ce[0]);
            if (lane == 31) {
                b0n = c0n = e0n = zero2();
                if (MULTI && strip + 1 < nstrips) {
                    const int slot = (strip + 1) * S;
                    const RowCoef a = row_coef(T, B, off_a, len_a, slot - task.pad_a);
                    const RowCoef b = row_coef(T, B, off_b, rb >= 0 ? len_b : 0, slot - task.pad_b);
                    b0n = make_float2(a.b, b.b);
                    c0n = make_float2(a.c, b.c);
                    e0n = make_float2(a.e, b.e);
                }
            }
            __syncwarp();
            float2 Mp[K], Ip[K], Dp[K];
#pragma unroll
            for (int k = 0; k < K; ++k) Mp[k] = Ip[k] = Dp[k] = zero2();
            float2 gW = zero2();   // row 0's M~ inner sum consumed this step (the diagonal input of row 0)
            float2 w0 = zero2();   // lane 0, strip 0: the row-0 boundary's inner sum c_0 X
            // Lane l runs column s - 2l at step s (a skew of two columns per lane), so what lane l-1 hands over
            // at the end of a step is shuffled at the start of the next one and consumed a step later: the
            // shuffle's latency is off the per-step chain (the I~ recurrence down the lane's rows).
            float2 pendV = zero2();                     // I~ of row 0 for next step's column
            float2 pendW1 = zero2(), pendW2 = zero2();  // row 0's M~ inner sums for the next two steps
            int hap = task.hap_begin - 1;
            const bool last_strip = (strip == nstrips - 1);
            float2 nxV = zero2(), nxW = zero2(), l0W = zero2();  // strip boundary (MULTI, lane 0): prefetched
            if (MULTI && strip > 0 && lane == 0 && ncols > 0) {
                nxV = scratch[0];
                nxW = scratch[1];
            }
            float2 sV = zero2(), sW = zero2();  // what this lane hands the lane below at the end of a step
            const int nsteps = ncols + 62;
            // column code of the next step, loaded one step ahead (the code plane has kCodePad bytes on
            // both sides, so columns just outside the stream are readable; CHK steps mask them)
            uint32_t code_next = (uint32_t)__ldg(stream - 2 * lane);
            // One wavefront step.  CHK steps handle columns outside the stream (lanes that have not started
            // or have finished), haplotype starts (state reset) and ends (lane 31 emits); they are needed
            // only in the 63 steps after each haplotype start, where those events fall.  Every other step
            // runs the check-free form.
            auto step = [&](const int s, auto chk_tag) {
                constexpr bool CHK = decltype(chk_tag)::value;
                const int c = s - 2 * lane;
                bool valid = true;
                uint32_t code = code_next;
                code_next = (uint32_t)__ldg(stream + c + 1);
                if constexpr (CHK) {
                    valid = (c >= 0) && (c < ncols);
                    code = valid ? code : 0u;
                }
                // Lane l-1's hand-over from its last step (its column c + 1): shuffled now, consumed next step
                // (I~) and the step after (the inner sum for column c + 2).  Shuffled before this lane resets its
                // own state at a haplotype start, since lane l+1 still needs this lane's previous column.
                const float2 shV = shfl_up2(sV);
                const float2 shW = shfl_up2(sW);
                float2 uV = pendV;  // I~ of this lane's row 0 at this column
                gW = pendW2;        // row 0's M~ inner sum for this column
                pendV = shV;
                pendW2 = pendW1;
                pendW1 = shW;
                // lane 0 takes the row-0 boundary (strip 0) or the previous strip's last row instead
                // (selects on the ALU pipe, not multiplies on the FMA pipe)
                if (MULTI && strip > 0) {
                    if (lane == 0) {
                        uV = nxV;
                        gW = l0W;
                        l0W = nxW;
                        if (c + 1 < ncols) {
                            nxV = scratch[2 * (c + 1) + 0];
                            nxW = scratch[2 * (c + 1) + 1];
                        }
                    }
                } else if (lane == 0) {
                    uV = zero2();
                }
                if constexpr (CHK) {
                    if (code & kColFirst) {
                        ++hap;
                        const float init = __ldg(B.hap_init_f + hap);
                        const float2 X = make_float2(init, rb >= 0 ? init : 0.f);
                        // dummy rows (global slot < pad) hold the row-0 value X in D^; a pad may reach past
                        // strip 0 for the shorter read of a pair
                        const int slot0 = strip * S + lane * K;
#pragma unroll
                        for (int k = 0; k < K; ++k) {
                            Mp[k] = Ip[k] = zero2();
                            Dp[k] = make_float2((slot0 + k < task.pad_a) ? X.x : 0.f, (slot0 + k < task.pad_b) ? X.y : 0.f);
                        }
                        const float2 gD = make_float2((slot0 - 1 < task.pad_a) ? X.x : 0.f,
                                                      (slot0 - 1 < task.pad_b) ? X.y : 0.f);
                        gW = mul2(cc[0], gD);
                        if (lane == 0 && strip == 0) w0 = mul2(cc[0], X);
                    }
                }
                if (!(MULTI && strip > 0) && lane == 0) gW = w0;
                const float4 *pri4 = prior_tbl4 + (code & 7u) * 32;
                float2 prs[2 * KP];
#pragma unroll
                for (int kk = 0; kk < KP; ++kk) {
                    const float4 v = pri4[kk * kBases * 32];
                    prs[2 * kk] = make_float2(v.x, v.y);
                    prs[2 * kk + 1] = make_float2(v.z, v.w);
                }
                // pass 1 (bottom-up so the row above is still the previous column): M and D^
#pragma unroll
                for (int k = K - 1; k >= 0; --k) {
                    const float2 pr = prs[k];
                    float2 Mn;
                    if (k) {
                        Mn = mul2(pr, fma2(Ip[k - 1], cb[k], fma2(Dp[k - 1], cc[k], Mp[k - 1])));
                    } else {
                        Mn = mul2(pr, gW);
                    }
                    const float2 Dn = fma2(Dp[k], cdd[k], Mp[k]);
                    Mp[k] = Mn;
                    Dp[k] = Dn;
                }
                // pass 2 (top-down): I~ from the row above at this column; row 0's comes from the lane above
                Ip[0] = uV;
#pragma unroll
                for (int k = 1; k < K; ++k) Ip[k] = fma2(Ip[k - 1], ce[k], Mp[k - 1]);
                const float2 i_acc = Ip[K >= 2 ? K - 2 : 0];  // I~(R+1) at this column (K >= 2)
                // hand the lane below its row 0's I~ at this column and M~ inner sum for the next
                sV = fma2(Ip[K - 1], e0n, Mp[K - 1]);
                sW = fma2(Ip[K - 1], b0n, fma2(Dp[K - 1], c0n, Mp[K - 1]));
                if (last_strip) {
                    if constexpr (CHK) {
                        if (lane == 31 && (code & kColLast)) {
                            const float2 t = add2(add2(Dp[K - 1], Mp[K - 1]), i_acc);
                            emit_fp32(B, t.x, __ldg(B.read_scale + ra), ra, hap, out_a + hap);
                            if (rb >= 0) emit_fp32(B, t.y, __ldg(B.read_scale + rb), rb, hap, out_b + hap);
                        }
                    }
                } else if (MULTI && lane == 31 && valid) {
                    scratch[2 * c + 0] = sV;
                    scratch[2 * c + 1] = sW;
                }
            };
            // haplotype boundaries of this task: columns hb(j) = hap_off[hap_begin + j] - col0, hb(n) = ncols
            const int64_t *hoff = B.hap_off + task.hap_begin;
            const int nh_task = task.hap_end - task.hap_begin;
            int s = 0, j = 0;
            while (s < nsteps) {
                while (j <= nh_task && (int)(hoff[j] - col0) <= s) ++j;
                const int window_end = min((int)(hoff[j - 1] - col0) + 63, nsteps);
                // unrolled (4 checked, 16 check-free steps; measured best of 2-32): the scheduler interleaves
                // one step's I~ chain and shuffles with the following steps' M~ and D~
                if (s < window_end) {
#pragma unroll 4
                    for (; s < window_end; ++s) step(s, std::true_type{});
                    continue;
                }
                const int next_boundary = (j <= nh_task) ? (int)(hoff[j] - col0) : nsteps;
#pragma unroll 16
                for (; s < next_boundary; ++s) step(s, std::false_type{});
            }
            if (MULTI) __syncwarp();
        }
    }
}

// Per read: log2 a_R = sum over its positions of -log2 MM (the FP32 pass's row rescaling, with the float
// matchToMatch values its coefficients use, from a host-built FP64 table), summed in FP64 in an order fixed by the
// read alone, so that a read's
// result does not depend on the task, rows per lane or batch it runs in.  Stored as (2^-(la - n), n), n = round(la).
// One warp per read; computed once per upload (after the read preparation for raw batches).
__global__ void read_scale_kernel(DevTables T, DevBatch B, int64_t n_reads, float2 *scale) {
    const int lane = threadIdx.x & 31;
    for (int64_t r = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < n_reads;
         r += ((int64_t)gridDim.x * blockDim.x) >> 5) {
        const int64_t off = B.read_off[r], len = B.read_off[r + 1] - off;
        double la = 0.0;
        for (int64_t p = lane; p < len; p += 32)
            la += __ldg(T.lm2m_d + B.ins[off + p] * 128 + B.dels[off + p]);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) la += __shfl_xor_sync(kFull, la, o);
        if (lane == 0) {
            const double n = rint(la);
            scale[r] = make_float2((float)exp2(n - la), (float)n);
        }
    }
}

// Final log10 un-scaling of the FP32 pass, in FP64: out = log10(t) - log10(a_R) - log10(2^120).  Runs before the FP64
// queue kernel, which then overwrites the pairs it recomputes (their slots hold no accepted sum).
__global__ void finalize_fp32_kernel(double *out, const int64_t *n_out) {
    const int64_t n = *n_out;
    const double log10_2 = 0.30102999566398120;
    for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const float2 v = reinterpret_cast<const float2 *>(out)[i];  // (t, log2 a_R), see emit_fp32
        out[i] = log10((double)v.x) - (double)v.y * log10_2 - kLog10Scale32;
    }
}

// ---------------------------------------------------------------------------------------------------
// FP64 wavefront, one (read, haplotype) pair per warp, K rows per lane, strips of 32*K rows, in two tiers.
//
// RESCALED (queue 1: host-routed pairs and FP32 underflows): the FP32 kernel's rescaled recurrence in FP64,
// 5 DP operations per cell instead of 8 (the FP64 pipe runs at 1/64 of the FP32 rate on this part):
//    M~ = prior * fma(I~_diag, b_i, fma(D~_diag, c_i, M~_diag)),  I~ = fma(I~_up, e_i, M~_up),
//    D~ = fma(D~_left, DD_i, M~_left),  sum over the haplotype of M~_R + (MI_R / MM_R) I~_R.
// The scale is S' = 2^960 instead of 2^1020 (headroom for I~ and D~, which carry 1 / MI and 1 / MD), and the
// initial condition is divided by 2^round(la), la = log2 a_R = sum of -log2 MM_i, so that the last row sits at
// scale S' like the unscaled recurrence.  Along every contributing path the rescaled states stay above the
// final sum's magnitude, so a result of log10 L >= kRescaledFloor (well inside the FP64 range at S') is as
// accurate as the unscaled recurrence; lower or non-finite results go to queue 2.
//
// EXACT (queue 2: those, and reads the host marks, e.g. matchToMatch ~ 0): the unscaled recurrence with the
// reference's 2^1020 initial condition, so it underflows exactly where LoglessPairHMM does.
constexpr double kLog10Scale64R = 288.9887958374219;  // log10(2^960)
constexpr double kRescaledFloor = GHMM_FP64_RESCALED_FLOOR;

template <int K, bool RESCALED>
__global__ void __launch_bounds__(128) fp64_queue_kernel(DevTables T, DevBatch B) {
    constexpr int S = 32 * K;
    const int lane = threadIdx.x & 31;
    const int64_t warp_global = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    double *scratch = B.scratch64 + warp_global * B.scratch64_cols * 3;
    const PairRef *queue = RESCALED ? B.rerun : B.rerun + B.rerun_capacity;
    const int total = min(B.counters[RESCALED ? 1 : 4], (int)B.rerun_capacity);
    const int cursor = RESCALED ? 2 : 5;
    for (;;) {
        int t = 0;
        if (lane == 0) t = atomicAdd(&B.counters[cursor], 1);
        t = __shfl_sync(kFull, t, 0);
        if (t >= total) break;
        const PairRef pr = queue[t];
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
        // RESCALED: la = log2 a_R, and the initial condition divided by 2^round(la)
        double la = 0.0, init = B.hap_init_d[hap];
        if (RESCALED) {
            for (int p = lane; p < R; p += 32) {
                const uint8_t ins = B.ins[roff + p], del = B.dels[roff + p];
                la -= log2(__ldg(T.m2m_d + ins * 128 + del));
            }
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) la += __shfl_xor_sync(kFull, la, o);
            init = scalbn(init, -60 - (int)rint(la));
        }
        const int nstrips = (R + S - 1) / S;
        const int pad = nstrips * S - R;
        const uint8_t *hb = B.hap_bases + hoff;
        double acc = 0.0, kappa = 0.0;
        if (RESCALED) {
            const uint8_t ins = B.ins[roff + R - 1], del = B.dels[roff + R - 1];
            kappa = __ldg(T.err_d + ins) / __ldg(T.m2m_d + ins * 128 + del);
        }
        for (int strip = 0; strip < nstrips; ++strip) {
            // per-row coefficients: RESCALED (b, c, e, DD); exact (MM, IM, MI, II, MD)
            double pm[K], pe[K], c1[K], c2[K], c3[K], c4[K], c5[K];
            uint32_t rbase[K];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const int p = strip * S + lane * K + k - pad;
                if (p < 0) {
                    pm[k] = pe[k] = 0.0;
                    c1[k] = c2[k] = c3[k] = c5[k] = 0.0;
                    c4[k] = RESCALED ? 1.0 : 0.0;  // DD = 1 keeps a dummy row's D~ at the row-0 value
                    rbase[k] = 0x100u;  // matches nothing
                } else {
                    const uint8_t base = B.bases[roff + p], q = B.quals[roff + p];
                    const uint8_t ins = B.ins[roff + p], del = B.dels[roff + p], gcp = B.gcp[roff + p];
                    pm[k] = __ldg(T.prob_d + q);
                    pe[k] = base == 'N' ? pm[k] : __ldg(T.err3_d + q);
                    const double mm = __ldg(T.m2m_d + ins * 128 + del), im = __ldg(T.prob_d + gcp);
                    const double mi = __ldg(T.err_d + ins), ii = __ldg(T.err_d + gcp), md = __ldg(T.err_d + del);
                    if (RESCALED) {
                        double mm_p = 1.0, mi_p = 1.0, md_p = 1.0;
                        if (p > 0) {
                            const uint8_t ins_p = B.ins[roff + p - 1], del_p = B.dels[roff + p - 1];
                            mm_p = __ldg(T.m2m_d + ins_p * 128 + del_p);
                            mi_p = __ldg(T.err_d + ins_p);
                            md_p = __ldg(T.err_d + del_p);
                        }
                        c1[k] = im * mi_p / (mm * mm_p);                  // b
                        c2[k] = im * md_p / mm;                           // c
                        c3[k] = (p > 0) ? ii * mi_p / (mi * mm_p) : 0.0;  // e
                        c4[k] = ii;                                       // DD
                        c5[k] = 0.0;
                    } else {
                        c1[k] = mm;
                        c2[k] = im;
                        c3[k] = mi;
                        c4[k] = ii;
                        c5[k] = md;
                    }
                    rbase[k] = base;
                }
            }
            double Mp[K], Ip[K], Dp[K];
#pragma unroll
            for (int k = 0; k < K; ++k) {
                const bool dummy = (strip == 0) && (lane * K + k < pad);
                Mp[k] = Ip[k] = 0.0;
                Dp[k] = dummy ? init : 0.0;
            }
            // exact: DD of dummy rows is 1 so their D stays at the row-0 value
            double tdd[K];
#pragma unroll
            for (int k = 0; k < K; ++k) tdd[k] = ((strip == 0) && (lane * K + k < pad)) ? 1.0 : c4[k];
            double gM = 0.0, gI = 0.0;
            double gD = ((strip == 0) && (lane * K - 1 < pad)) ? init : 0.0;
            const double bnd = (strip == 0) ? init : 0.0;
            const bool last_strip = strip == nstrips - 1;
            double nxM = 0.0, nxI = 0.0, nxD = 0.0;
            if (strip > 0 && lane == 0) {
                nxM = scratch[0];
                nxI = scratch[1];
                nxD = scratch[2];
            }
            const int nsteps = H + 31;
            for (int s = 0; s < nsteps; ++s) {
                const int c = s - lane;
                const bool valid = c >= 0 && c < H;
                const uint32_t y = valid ? (uint32_t)__ldg(hb + c) : 0x200u;
                const bool yn = (y == 'N');
                if (c == 0) {  // column-0 boundary (lanes compute ahead of their first column)
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        Mp[k] = Ip[k] = 0.0;
                        Dp[k] = ((strip == 0) && (lane * K + k < pad)) ? init : 0.0;
                    }
                    gM = gI = 0.0;
                    gD = ((strip == 0) && (lane * K - 1 < pad)) ? init : 0.0;
                }
                double uM = __shfl_up_sync(kFull, Mp[K - 1], 1);
                double uI = __shfl_up_sync(kFull, Ip[K - 1], 1);
                double uD = __shfl_up_sync(kFull, Dp[K - 1], 1);
                if (lane == 0) {
                    if (strip == 0) {
                        uM = 0.0;
                        uI = 0.0;
                        uD = bnd;
                    } else {
                        uM = nxM;
                        uI = nxI;
                        uD = nxD;
                        if (c + 1 < H) {
                            nxM = scratch[3 * (c + 1) + 0];
                            nxI = scratch[3 * (c + 1) + 1];
                            nxD = scratch[3 * (c + 1) + 2];
                        }
                    }
                }
#pragma unroll
                for (int k = K - 1; k >= 0; --k) {
                    const double dM = k ? Mp[k - 1] : gM;
                    const double dI = k ? Ip[k - 1] : gI;
                    const double dD = k ? Dp[k - 1] : gD;
                    const double prior = (rbase[k] == y || yn) ? pm[k] : pe[k];
                    double Mn, Dn;
                    if (RESCALED) {
                        Mn = prior * fma(dI, c1[k], fma(dD, c2[k], dM));
                        Dn = fma(Dp[k], tdd[k], Mp[k]);
                    } else {  // the reference's grouping: prior x (M x MM + (I + D) x IM), so results deep in the
                              // subnormal range round as LoglessPairHMM's do
                        Mn = prior * fma(dM, c1[k], (dI + dD) * c2[k]);
                        Dn = fma(Dp[k], tdd[k], Mp[k] * c5[k]);
                    }
                    Mp[k] = Mn;
                    Dp[k] = Dn;
                }
                double aM = uM, aI = uI;
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    const double In = RESCALED ? fma(aI, c3[k], aM) : fma(aI, c4[k], aM * c3[k]);
                    Ip[k] = In;
                    aM = Mp[k];
                    aI = In;
                }
                gM = uM;
                gI = uI;
                gD = uD;
                if (valid && lane == 31) {
                    if (last_strip) {
                        acc += RESCALED ? fma(kappa, Ip[K - 1], Mp[K - 1]) : Mp[K - 1] + Ip[K - 1];
                    } else {
                        scratch[3 * c + 0] = Mp[K - 1];
                        scratch[3 * c + 1] = Ip[K - 1];
                        scratch[3 * c + 2] = Dp[K - 1];
                    }
                }
            }
            __syncwarp();
        }
        if (lane == 31) {
            if (RESCALED) {
                const double rla = rint(la);
                const double v = log10(acc) - kLog10Scale64R - (la - rla) * 0.30102999566398120;
                if (v >= kRescaledFloor && v <= 0.0) {
                    B.out[out_index] = v;
                } else {  // too close to the FP64 range at S' (or not finite): the exact tier recomputes it
                    const int idx = atomicAdd(&B.counters[4], 1);
                    if ((int64_t)idx < B.rerun_capacity)
                        B.rerun[B.rerun_capacity + idx] = pr;
                    else
                        atomicExch(&B.counters[3], 1);
                }
            } else {
                B.out[out_index] = log10(acc) - kLog10Scale64;
            }
        }
    }
}

// ---------------------------------------------------------------------------------------------------
// Plain FP64 form: one (read, haplotype) pair per 256-thread block; thread t owns rows t+1+256m (m<ROWS:
// 4 rows for reads up to 1024 bases, 8 up to 2048); three rolling anti-diagonals of M, I, D in shared
// memory; one barrier per diagonal; Java's order of operations (no fused multiply-add), so the sums equal
// the FP64 oracle's.
constexpr int kPlainThreads = 256;

template <int kPlainRows>
__global__ void __launch_bounds__(kPlainThreads) plain_fp64_kernel(DevTables T, DevBatch B, int region, int nh) {
    extern __shared__ double sm[];
    const int pair = blockIdx.x;
    const int64_t read = B.region_read_off[region] + pair / nh;
    const int64_t hap = B.region_hap_off[region] + pair % nh;
    const int64_t roff = B.read_off[read];
    const int R = (int)(B.read_off[read + 1] - roff);
    const int64_t hoff = B.hap_off[hap];
    const int H = (int)(B.hap_off[hap + 1] - hoff);
    const int64_t out_index = B.out_off[region] + pair;
    if (R == 0 || H == 0) {
        if (threadIdx.x == 0) B.out[out_index] = -INFINITY;
        return;
    }
    const int W = R + 1;
    double *Mb = sm, *Ib = sm + 3 * W, *Db = sm + 6 * W;  // [3][W] each
    const double init = B.hap_init_d[hap];
    double t_mm[kPlainRows], t_im[kPlainRows], t_mi[kPlainRows], t_ii[kPlainRows], t_md[kPlainRows];
    double p_m[kPlainRows], p_e[kPlainRows];
    uint8_t xb[kPlainRows];
#pragma unroll
    for (int m = 0; m < kPlainRows; ++m) {
        const int i = threadIdx.x + 1 + m * kPlainThreads;
        if (i <= R) {
            const int p = i - 1;
            const uint8_t q = B.quals[roff + p], ins = B.ins[roff + p], del = B.dels[roff + p];
            const uint8_t gcp = B.gcp[roff + p];
            t_mm[m] = T.m2m_d[ins * 128 + del];
            t_im[m] = T.prob_d[gcp];
            t_mi[m] = T.err_d[ins];
            t_ii[m] = T.err_d[gcp];
            t_md[m] = T.err_d[del];
            p_m[m] = T.prob_d[q];
            p_e[m] = T.err3_d[q];
            xb[m] = B.bases[roff + p];
        } else {
            t_mm[m] = t_im[m] = t_mi[m] = t_ii[m] = t_md[m] = p_m[m] = p_e[m] = 0.0;
            xb[m] = 0;
        }
    }
    for (int b = 0; b < 3; ++b)
        for (int i = threadIdx.x; i < W; i += kPlainThreads) {
            Mb[b * W + i] = 0.0;
            Ib[b * W + i] = 0.0;
            Db[b * W + i] = (i == 0) ? init : 0.0;
        }
    __syncthreads();
    double sum = 0.0;
    for (int d = 2; d <= R + H; ++d) {
        const int cur = d % 3, p1 = (d + 2) % 3, p2 = (d + 1) % 3;
#pragma unroll
        for (int m = 0; m < kPlainRows; ++m) {
            const int i = threadIdx.x + 1 + m * kPlainThreads;
            if (i > R) continue;
            const int j = d - i;
            if (j == 0) {  // column-0 boundary
                Mb[cur * W + i] = 0.0;
                Ib[cur * W + i] = 0.0;
                Db[cur * W + i] = 0.0;
                continue;
            }
            if (j < 1 || j > H) continue;
            const uint8_t y = B.hap_bases[hoff + j - 1];
            const double prior = (xb[m] == y || xb[m] == 'N' || y == 'N') ? p_m[m] : p_e[m];
            const double mdiag = Mb[p2 * W + i - 1], idiag = Ib[p2 * W + i - 1], ddiag = Db[p2 * W + i - 1];
            const double mup = Mb[p1 * W + i - 1], iup = Ib[p1 * W + i - 1];
            const double mleft = Mb[p1 * W + i], dleft = Db[p1 * W + i];
            const double mv = __dmul_rn(prior, __dadd_rn(__dadd_rn(__dmul_rn(mdiag, t_mm[m]), __dmul_rn(idiag, t_im[m])),
                                                         __dmul_rn(ddiag, t_im[m])));
            const double iv = __dadd_rn(__dmul_rn(mup, t_mi[m]), __dmul_rn(iup, t_ii[m]));
            const double dv = __dadd_rn(__dmul_rn(mleft, t_md[m]), __dmul_rn(dleft, t_ii[m]));
            Mb[cur * W + i] = mv;
            Ib[cur * W + i] = iv;
            Db[cur * W + i] = dv;
            if (i == R) sum = __dadd_rn(sum, __dadd_rn(mv, iv));
        }
        __syncthreads();
    }
    if ((int)threadIdx.x == (R - 1) % kPlainThreads) B.out[out_index] = log10(sum) - kLog10Scale64;
}

// ---------------------------------------------------------------------------------------------------
// FP32 / FP64 pipe peak probes: register-resident chains, 8 independent per thread.
template <int N>
__global__ void peak_ffma_kernel(float *out, int iters, float x, float y) {
    float a[N];
#pragma unroll
    for (int i = 0; i < N; ++i) a[i] = threadIdx.x * 1e-7f + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < N; ++i) a[i] = fmaf(a[i], x, y);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i) s += a[i];
    if (s == 12345.678f) out[threadIdx.x] = s;
}

template <int N>
__global__ void peak_ffma2_kernel(float *out, int iters, float x, float y) {
    float2 a[N];
#pragma unroll
    for (int i = 0; i < N; ++i) a[i] = make_float2(threadIdx.x * 1e-7f + i, threadIdx.x * 2e-7f + i);
    const float2 xx = make_float2(x, x), yy = make_float2(y, y);
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < N; ++i) a[i] = __ffma2_rn(a[i], xx, yy);
    }
    float s = 0.f;
#pragma unroll
    for (int i = 0; i < N; ++i) s += a[i].x + a[i].y;
    if (s == 12345.678f) out[threadIdx.x] = s;
}

template <int N>
__global__ void peak_dfma_kernel(double *out, int iters, double x, double y) {
    double a[N];
#pragma unroll
    for (int i = 0; i < N; ++i) a[i] = threadIdx.x * 1e-7 + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < N; ++i) a[i] = fma(a[i], x, y);
    }
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) s += a[i];
    if (s == 12345.678) out[threadIdx.x] = s;
}

// ---------------------------------------------------------------------------------------------------
static size_t fp32_smem_bytes(int k, int block) { return (size_t)(block / 32) * ((k + 1) / 2) * kBases * 32 * sizeof(float4); }

template <int K, bool MULTI>
static int launch_fp32_k(const DevTables &t, const DevBatch &b, int grid, int block, cudaStream_t s) {
    const size_t smem = fp32_smem_bytes(K, block);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(fp32_bucket_kernel<K, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    fp32_bucket_kernel<K, MULTI><<<grid, block, smem, s>>>(t, b);
    return (int)cudaGetLastError();
}

int launch_fp32_bucket(const DevTables &t, const DevBatch &b, int k, int grid, int block, cudaStream_t s) {
    // k encodes rows per lane in the low 4 bits and the multi-strip flag in bit 4
    const bool multi = (k & 16) != 0;
    switch (k & 15) {
#define GHMM_CASE(KK)                                                                                   \
    case KK:                                                                                            \
        return multi ? launch_fp32_k<KK, true>(t, b, grid, block, s) : launch_fp32_k<KK, false>(t, b, grid, block, s);
        GHMM_CASE(1)
        GHMM_CASE(2)
        GHMM_CASE(3)
        GHMM_CASE(4)
        GHMM_CASE(5)
        GHMM_CASE(6)
        GHMM_CASE(7)
        GHMM_CASE(8)
#undef GHMM_CASE
        default:
            return (int)cudaErrorInvalidValue;
    }
}

int fp32_kernel_occupancy(int k, int block, int *blocks_per_sm) {
    const bool multi = (k & 16) != 0;
    cudaError_t e = cudaErrorInvalidValue;
    switch (k & 15) {
#define GHMM_OCC(KK)                                                                                              \
    case KK:                                                                                                      \
        e = multi ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fp32_bucket_kernel<KK, true>, block,  \
                                                                  fp32_smem_bytes(KK, block))                          \
                  : cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fp32_bucket_kernel<KK, false>, block, \
                                                                  fp32_smem_bytes(KK, block));                         \
        break;
        GHMM_OCC(1)
        GHMM_OCC(2)
        GHMM_OCC(3)
        GHMM_OCC(4)
        GHMM_OCC(5)
        GHMM_OCC(6)
        GHMM_OCC(7)
        GHMM_OCC(8)
#undef GHMM_OCC
        default:
            break;
    }
    return (int)e;
}

int launch_fp64_queue(const DevTables &t, const DevBatch &b, int grid, int block, cudaStream_t s) {
    fp64_queue_kernel<kMaxK64, true><<<grid, block, 0, s>>>(t, b);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return (int)e;
    fp64_queue_kernel<kMaxK64, false><<<grid, block, 0, s>>>(t, b);
    return (int)cudaGetLastError();
}

int launch_read_scale(const DevTables &t, const DevBatch &b, int64_t n_reads, float2 *scale, int sm_count,
                      cudaStream_t s) {
    if (n_reads <= 0) return 0;
    const int64_t want = (n_reads + 7) / 8;  // 8 warps per 256-thread block
    read_scale_kernel<<<(int)(want < (int64_t)sm_count * 8 ? want : (int64_t)sm_count * 8), 256, 0, s>>>(t, b, n_reads,
                                                                                                          scale);
    return (int)cudaGetLastError();
}

int launch_finalize_fp32(double *out, const int64_t *n_out, int sm_count, cudaStream_t s) {
    finalize_fp32_kernel<<<sm_count * 4, 256, 0, s>>>(out, n_out);
    return (int)cudaGetLastError();
}

int fp64_kernel_occupancy(int block, int *blocks_per_sm) {
    // both tiers run on the same grid and scratch: the smaller occupancy of the two
    int a = 0, b = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&a, fp64_queue_kernel<kMaxK64, true>, block, 0);
    if (e != cudaSuccess) return (int)e;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, fp64_queue_kernel<kMaxK64, false>, block, 0);
    *blocks_per_sm = a < b ? a : b;
    return (int)e;
}

// Shared memory: three diagonals of M, I, D over R+1 rows, sized by the region's longest read.
int launch_plain_region(const DevTables &t, const DevBatch &b, int region, int n_reads, int n_haps,
                              int max_read_len, cudaStream_t s) {
    if (n_reads <= 0 || n_haps <= 0) return 0;
    if (max_read_len > kPlainMaxRead) return (int)cudaErrorInvalidValue;
    const size_t smem = sizeof(double) * 9 * (size_t)(max_read_len + 1);
    const bool wide = max_read_len > 4 * kPlainThreads;
    if (smem > 48 * 1024) {
        cudaError_t e = wide ? cudaFuncSetAttribute(plain_fp64_kernel<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)
                             : cudaFuncSetAttribute(plain_fp64_kernel<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    if (wide)
        plain_fp64_kernel<8><<<n_reads * n_haps, kPlainThreads, smem, s>>>(t, b, region, n_haps);
    else
        plain_fp64_kernel<4><<<n_reads * n_haps, kPlainThreads, smem, s>>>(t, b, region, n_haps);
    return (int)cudaGetLastError();
}

int measure_peaks_device(int sm_count, double *fp32, double *fp32x2, double *fp64, cudaStream_t s) {
    float *fo = nullptr;
    double *dout = nullptr;
    if (cudaMalloc(&fo, 1024 * sizeof(float)) != cudaSuccess) return (int)cudaErrorMemoryAllocation;
    if (cudaMalloc(&dout, 1024 * sizeof(double)) != cudaSuccess) {
        cudaFree(fo);
        return (int)cudaErrorMemoryAllocation;
    }
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int block = 256, grid = sm_count * 8;
    constexpr int N = 8;
    const double threads = (double)grid * block;
    float ms = 0.f;
    int err = 0;
    // best of three timed launches after a warm-up, so a clock still ramping up does not lower the peak
    auto timeit = [&](auto launch, int iters, double flops_per_iter_thread, double *res) {
        launch(iters / 8);
        double best = 0.0;
        for (int rep = 0; rep < 3; ++rep) {
            cudaEventRecord(e0, s);
            launch(iters);
            cudaEventRecord(e1, s);
            cudaEventSynchronize(e1);
            cudaEventElapsedTime(&ms, e0, e1);
            const double v = threads * iters * flops_per_iter_thread / (ms * 1e-3) / 1e12;
            if (v > best) best = v;
        }
        if (res) *res = best;
        if (cudaGetLastError() != cudaSuccess) err = 1;
    };
    timeit([&](int it) { peak_ffma_kernel<N><<<grid, block, 0, s>>>(fo, it, 0.999999f, 1e-6f); }, 1 << 16,
           2.0 * N, fp32);
    timeit([&](int it) { peak_ffma2_kernel<N><<<grid, block, 0, s>>>(fo, it, 0.999999f, 1e-6f); }, 1 << 15,
           4.0 * N, fp32x2);
    timeit([&](int it) { peak_dfma_kernel<N><<<grid, block, 0, s>>>(dout, it, 0.999999, 1e-6); }, 1 << 11,
           2.0 * N, fp64);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(fo);
    cudaFree(dout);
    return err ? (int)cudaErrorLaunchFailure : 0;
}

}  // namespace ghmm
