// pd_packed.cu -- the FP32 PD-HMM forward in the layout of the regular FP32 pass.
//
// LoglessPDPairHMM (src/main/java/org/broadinstitute/hellbender/utils/pairhmm/LoglessPDPairHMM.java:35-150) adds
// three branch matrices bM, bI, bD to LoglessPairHMM's M, I, D.  Along a row, the state a column is processed in
// (NORMAL, INSIDE_DEL, AFTER_DEL, set by the PD flags of the columns before it) decides:
//    NORMAL:     bX(i,j) = X(i,j-1)
//    INSIDE_DEL: bX(i,j) = bX(i,j-1)
//    AFTER_DEL:  bX(i,j) = max(bX(i,j-1), X(i,j-1)), and M and D read max(bX, X) of their diagonal / left inputs
// and at a DEL_END column I reads max(bX, X) of the row above.  An undetermined SNP column also matches a read
// base against its alternative (isBasePDMatching, :196-210).
//
// pd_bucket_kernel<K> runs these pairs as the regular FP32 pass does (fp32_bucket_kernel in kernels.cu, whose
// header comment describes the layout): read-pair tasks of two reads of one region in the halves of float2, K rows
// per lane, the region's haplotypes streamed back to back, the two-column lane skew with its hand-over of row 0's
// I~ and M~ inner sum, rescaled rows, the per-warp prior table and the accumulator rows.  Rescaling a row by a
// positive factor commutes with max, so the branch states live in the same rescaled form as the states they copy.
//
// The PD work is per column, from an op byte the host derives from the flags (pd_host.cpp):
//  * kPdOpCopy: store the column's branch states, only where a later column reads them (the column before a
//    deletion's INSIDE_DEL or AFTER_DEL columns, or a DEL_END column): bX(j) = X(j-1) at a NORMAL column.  Elsewhere
//    the branch states go stale and nothing reads them, so most columns do no branch work at all.
//  * kPdOpAfter: the previous column's M, I, D of every row are replaced by max(bX, X) before the step (every use
//    of them in an AFTER_DEL column is that max); with kPdOpCopy the branch states take the same values.
//  * kPdOpDelEnd: I of rows 1..K-1 reads max(bX, X) of the row above; row 0's I~ comes from the lane above, which
//    applies the max in its hand-over at this column.
//  * kPdOpNextAfter: the next column is AFTER_DEL, so the lane's hand-over of row 0's M~ inner sum for it (the
//    lane below's diagonal input there) uses max(bX, X) of its last row.
//  * kPdOpSnp (alternative base in bits 5-6): the prior is the match prior when the read base equals the column's
//    base or the alternative (or is N), picked from three rows of the prior table without a per-row base compare;
//    with kPdOpSnpAllBut, three bases match (two alternatives) and bits 5-6 name the fourth.  A column whose
//    alternatives cover all four bases carries the code of N (pd_host.cpp), which matches every read base.
// These run only in lanes at such columns (lane-divergent branches), and only in steps where some lane of the warp
// is at such a column (a warp vote; the other steps are the regular kernel's).  The accumulator rows below each read
// never take a branch state (theirs stay 0, so max(bX, X) = X for them), and the first accumulator row's I never
// takes the DEL_END max, since it sums the read's last row rather than stepping the recurrence.
//
// Reads longer than 32 K - 2 rows run in strips as in the regular kernel: lane 31 of a strip stores per column its
// hand-over to the row below (with the PD max where the column asks for it) for lane 0 of the next strip; the
// accumulator rows and their exclusions belong to the last strip.  The host sends a region to the general PD kernel
// (pd.cu) instead when a haplotype leaves a deletion open at its last column (the later rows would start INSIDE_DEL,
// the first row NORMAL); reads the regular routing sends to FP64 go there too.  A sum below
// GHMM_FP32_RERUN_THRESHOLD (or not finite) queues the pair for the FP64 PD kernel.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <type_traits>

#include "../../include/ghmm.h"
#include "fp32_rows.cuh"
#include "ghmm_internal.h"

namespace ghmm {
namespace {

// max that returns NaN when either input is NaN (Java's Math.max), so a non-finite state reaches the sum and the
// pair's rerun instead of being dropped by maxNum
__device__ __forceinline__ float max_nan(float a, float b) {
    float r;
    asm("max.NaN.f32 %0, %1, %2;" : "=f"(r) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ float2 max2(float2 a, float2 b) { return make_float2(max_nan(a.x, b.x), max_nan(a.y, b.y)); }

// The match prior of an undetermined SNP column from the prior table rows of its base (t1), its alternative (t2)
// and a third base (t3): t1 and t2 differ only for a read base equal to one of the two, and then the one that is the
// match prior is t1 when t1 differs from the mismatch prior t3, else t2.
__device__ __forceinline__ float snp_prior(float t1, float t2, float t3) { return (t1 == t2 || t1 != t3) ? t1 : t2; }
// The same for a column where three bases match, from the rows of the one that does not (tu), of N (tn: always the
// match prior) and of a matching base (tw): the read base is the non-matching one exactly when tu equals tn, and tw is
// then the mismatch prior (for a read N both are the match prior, which its row carries as both priors).
__device__ __forceinline__ float all_but_prior(float tu, float tn, float tw) { return tu == tn ? tw : tn; }

// Accepted sums as the regular pass stores them (raw (t s, n), turned into log10 by finalize_fp32_kernel); the
// rest queue for the FP64 PD kernel at rerun[rerun_capacity..).
__device__ __forceinline__ void emit_pd(const DevBatch &B, float t, float2 scale, int read, int hap,
                                        int64_t out_index) {
    t *= scale.x;
    const float la = scale.y;
    if (t > 0.f && t <= FLT_MAX && log2f(t) - la >= kLog2Threshold) {
        reinterpret_cast<float2 *>(B.out)[out_index] = make_float2(t, la);
    } else {
        const int idx = atomicAdd(&B.counters[kCounterPdRerun], 1);
        if ((int64_t)idx < B.rerun_capacity) {
            B.rerun[B.rerun_capacity + idx] = PairRef{read, hap};
        } else {
            atomicExch(&B.counters[3], 1);
        }
    }
}

// Blocks of 128 threads per SM ptxas is asked to fit: the branch registers (six floats per row) on top of the
// regular kernel's.
template <int K>
struct PdMinBlocks {
    static constexpr int value = 3;
};

template <int K, bool MULTI>
__global__ void __launch_bounds__(128, PdMinBlocks<K>::value) pd_bucket_kernel(DevTables T, DevBatch B,
                                                                             const uint8_t *ops_plane) {
    static_assert(K >= 2, "the accumulator rows need two rows of lane 31");
    constexpr int KEY = K | (MULTI ? 16 : 0);
    constexpr int S = 32 * K;
    const int task_begin = B.bucket_info[KEY], task_count = B.bucket_info[kNumBucketKeys + KEY];
    const int counter_slot = kCounterBucketBase + KEY;
    const int lane = threadIdx.x & 31;
    constexpr int KP = (K + 1) / 2;  // row pairs of the prior table
    extern __shared__ float4 pd_prior_smem4[];
    float4 *prior_tbl4 = pd_prior_smem4 + (size_t)(threadIdx.x >> 5) * (KP * kBases * 32) + lane;
    float2 *prior_tbl2 = reinterpret_cast<float2 *>(prior_tbl4);
    // branch states bM, bI, bD of the lane's rows, lane-private: [row][M, I, D][lane] after the 4 warps' tables
    float2 *bst = reinterpret_cast<float2 *>(pd_prior_smem4 + 4 * (KP * kBases * 32)) +
                  (size_t)(threadIdx.x >> 5) * (K * 3 * 32) + lane;
    // strip boundary of multi-strip tasks: per column lane 31's hand-over (I~ and the M~ inner sum) for lane 0 of
    // the next strip, as the regular kernel passes it
    float2 *scratch = nullptr;
    if (MULTI) scratch = B.scratch32 + (((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5) * B.scratch32_cols * 3;

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
        const uint8_t *opstream = ops_plane + col0;
        const int nstrips = MULTI ? task.nstrips : 1;

        for (int strip = 0; strip < nstrips; ++strip) {
            const bool last_strip = strip == nstrips - 1;
            const bool acc_lane = lane == 31 && last_strip;  // its last two rows are the accumulator rows of both reads
            float2 cb[K], cc[K], ce[K], cdd[K];
            __syncwarp();  // the previous task's (or strip's) steps have finished reading this warp's table
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
            float2 b0n = shfl_down2(cb[0]), c0n = shfl_down2(cc[0]), e0n = shfl_down2(ce[0]);
            if (lane == 31) {  // the row below lane 31: the next strip's first row, or none
                b0n = c0n = e0n = zero2();
                if (MULTI && !last_strip) {
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
            for (int k = 0; k < K; ++k) {
                Mp[k] = Ip[k] = Dp[k] = zero2();
                bst[(3 * k + 0) * 32] = bst[(3 * k + 1) * 32] = bst[(3 * k + 2) * 32] = zero2();
            }
            float2 gW = zero2(), w0 = zero2();
            float2 pendV = zero2(), pendW1 = zero2(), pendW2 = zero2();
            float2 sV = zero2(), sW = zero2();
            float2 nxV = zero2(), nxW = zero2(), l0W = zero2();  // lane 0 of a later strip: the strip above's hand-over
            if (MULTI && strip > 0 && lane == 0 && ncols > 0) {
                nxV = scratch[0];
                nxW = scratch[1];
            }
            int hap = task.hap_begin - 1;
            const int nsteps = ncols + 62;
            // code and op of the next step's column, loaded a step ahead (both planes have kCodePad zero bytes on
            // either side, so columns just outside the stream read as code 0 and no op)
            uint32_t code_next = (uint32_t)__ldg(stream - 2 * lane);
            uint32_t op_next = (uint32_t)__ldg(opstream - 2 * lane);
            auto step = [&](const int s, auto chk_tag) {
                constexpr bool CHK = decltype(chk_tag)::value;
                const int c = s - 2 * lane;
                uint32_t code = code_next, op = op_next;
                code_next = (uint32_t)__ldg(stream + c + 1);
                op_next = (uint32_t)__ldg(opstream + c + 1);
                bool valid = true;
                if constexpr (CHK) {
                    valid = (c >= 0) && (c < ncols);
                    code = valid ? code : 0u;
                    op = valid ? op : 0u;
                }
                const float2 shV = shfl_up2(sV);
                const float2 shW = shfl_up2(sW);
                float2 uV = pendV;
                gW = pendW2;
                pendV = shV;
                pendW2 = pendW1;
                pendW1 = shW;
                if (MULTI && strip > 0) {  // lane 0 takes the strip above's last row (W one step later, as it comes)
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
                        const int slot0 = strip * S + lane * K;
#pragma unroll
                        for (int k = 0; k < K; ++k) {
                            Mp[k] = Ip[k] = zero2();
                            Dp[k] = make_float2((slot0 + k < task.pad_a) ? X.x : 0.f,
                                                (slot0 + k < task.pad_b) ? X.y : 0.f);
                        }
                        const float2 gD = make_float2((slot0 - 1 < task.pad_a) ? X.x : 0.f,
                                                      (slot0 - 1 < task.pad_b) ? X.y : 0.f);
                        gW = mul2(cc[0], gD);
                        if (lane == 0 && strip == 0) w0 = mul2(cc[0], X);
                    }
                }
                if (!(MULTI && strip > 0) && lane == 0) gW = w0;
                auto body = [&](auto ops_tag) {
                    constexpr bool OPS = decltype(ops_tag)::value;
                    // branch states at this column, from the previous column's values (still in Mp, Ip, Dp)
                    if (OPS && (op & (kPdOpCopy | kPdOpAfter))) {
                        if (op & kPdOpAfter) {
#pragma unroll
                            for (int k = 0; k < K; ++k) {
                                Mp[k] = max2(bst[(3 * k + 0) * 32], Mp[k]);
                                Ip[k] = max2(bst[(3 * k + 1) * 32], Ip[k]);
                                Dp[k] = max2(bst[(3 * k + 2) * 32], Dp[k]);
                            }
                        }
                        if (op & kPdOpCopy) {  // (an AFTER_DEL column stores only when a later column reads it)
#pragma unroll
                            for (int k = 0; k < K; ++k) {
                                if (k >= K - 2 && acc_lane) continue;
                                bst[(3 * k + 0) * 32] = Mp[k];
                                bst[(3 * k + 1) * 32] = Ip[k];
                                bst[(3 * k + 2) * 32] = Dp[k];
                            }
                        }
                    }
                    const uint32_t ref = code & 7u;
                    const float4 *pri4 = prior_tbl4 + ref * 32;
                    float2 prs[2 * KP];
#pragma unroll
                    for (int kk = 0; kk < KP; ++kk) {
                        const float4 v = pri4[kk * kBases * 32];
                        prs[2 * kk] = make_float2(v.x, v.y);
                        prs[2 * kk + 1] = make_float2(v.z, v.w);
                    }
                    if (OPS && (op & kPdOpSnp)) {
                        const uint32_t alt = (op >> kPdOpAltShift) & 3u;
                        if (op & kPdOpSnpAllBut) {  // three bases match: all but `alt`
                            const uint32_t w = alt ? 0u : 1u;
                            const float4 *pu = prior_tbl4 + alt * 32, *pn = prior_tbl4 + 4 * 32;
                            const float4 *pw = prior_tbl4 + w * 32;
#pragma unroll
                            for (int kk = 0; kk < KP; ++kk) {
                                const float4 tu = pu[kk * kBases * 32], tn = pn[kk * kBases * 32];
                                const float4 tw = pw[kk * kBases * 32];
                                prs[2 * kk] =
                                    make_float2(all_but_prior(tu.x, tn.x, tw.x), all_but_prior(tu.y, tn.y, tw.y));
                                prs[2 * kk + 1] =
                                    make_float2(all_but_prior(tu.z, tn.z, tw.z), all_but_prior(tu.w, tn.w, tw.w));
                            }
                        } else {  // two bases match: the column's and `alt`
                            const uint32_t third = (uint32_t)__ffs(~((1u << ref) | (1u << alt))) - 1u;
                            const float4 *pa = prior_tbl4 + alt * 32, *pt = prior_tbl4 + third * 32;
#pragma unroll
                            for (int kk = 0; kk < KP; ++kk) {
                                const float4 t2 = pa[kk * kBases * 32], t3 = pt[kk * kBases * 32];
                                const float2 p0 = prs[2 * kk], p1 = prs[2 * kk + 1];
                                prs[2 * kk] = make_float2(snp_prior(p0.x, t2.x, t3.x), snp_prior(p0.y, t2.y, t3.y));
                                prs[2 * kk + 1] = make_float2(snp_prior(p1.x, t2.z, t3.z), snp_prior(p1.y, t2.w, t3.w));
                            }
                        }
                    }
                    // pass 1 (bottom-up): M~ and D~
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
                    // pass 2 (top-down): I~ from the row above at this column
                    Ip[0] = uV;
                    if (OPS && (op & kPdOpDelEnd)) {
#pragma unroll
                        for (int k = 1; k < K; ++k) {
                            float2 bi = bst[(3 * (k - 1) + 1) * 32], bm = bst[(3 * (k - 1) + 0) * 32];
                            // the first accumulator row sums row R as is
                            if (k == K - 2 && acc_lane) bi = bm = zero2();
                            Ip[k] = fma2(max2(bi, Ip[k - 1]), ce[k], max2(bm, Mp[k - 1]));
                        }
                    } else {
#pragma unroll
                        for (int k = 1; k < K; ++k) Ip[k] = fma2(Ip[k - 1], ce[k], Mp[k - 1]);
                    }
                    // hand-over to the lane below: row 0's I~ at this column and its M~ inner sum for the next column
                    float2 hI = Ip[K - 1], hM = Mp[K - 1];
                    // (K = 2: lane 31's row 0 in the last strip is an accumulator row, whose I takes no max)
                    if (OPS && (op & kPdOpDelEnd) && !(K == 2 && lane == 30 && last_strip)) {
                        hI = max2(bst[(3 * (K - 1) + 1) * 32], hI);
                        hM = max2(bst[(3 * (K - 1) + 0) * 32], hM);
                    }
                    sV = fma2(hI, e0n, hM);
                    float2 wI = Ip[K - 1], wD = Dp[K - 1], wM = Mp[K - 1];
                    if (OPS && (op & kPdOpNextAfter)) {
                        wI = max2(bst[(3 * (K - 1) + 1) * 32], wI);
                        wD = max2(bst[(3 * (K - 1) + 2) * 32], wD);
                        wM = max2(bst[(3 * (K - 1) + 0) * 32], wM);
                    }
                    sW = fma2(wI, b0n, fma2(wD, c0n, wM));
                    if (last_strip) {
                        if constexpr (CHK) {
                            if (lane == 31 && (code & kColLast)) {
                                const float2 i_acc = Ip[K - 2];  // I~(R+1) at this column
                                const float2 t2 = add2(add2(Dp[K - 1], Mp[K - 1]), i_acc);
                                emit_pd(B, t2.x, __ldg(B.read_scale + ra), ra, hap, out_a + hap);
                                if (rb >= 0) emit_pd(B, t2.y, __ldg(B.read_scale + rb), rb, hap, out_b + hap);
                            }
                        }
                    } else if (MULTI && lane == 31 && valid) {
                        scratch[2 * c + 0] = sV;
                        scratch[2 * c + 1] = sW;
                    }
                };
                // steps where no lane is at a column with PD work (about two in three) run the regular kernel's step,
                // without the op tests: 8 % faster than testing the op bits in every step
                if (__any_sync(kFull, op != 0u))
                    body(std::true_type{});
                else
                    body(std::false_type{});
            };
            // Step loops not unrolled: the lane-divergent op branches and the two step bodies behind the warp vote
            // split each step into several blocks anyway; unrolled 4 (checked) and 8 (check-free) the steps overflowed
            // the instruction cache (ncu: 6-8 cycles of "no instruction" stall per issue, half the speed), and with the
            // vote 2 (check-free) was still 4 % slower than 1
            const int64_t *hoff = B.hap_off + task.hap_begin;
            const int nh_task = task.hap_end - task.hap_begin;
            int s = 0, j = 0;
            while (s < nsteps) {
                while (j <= nh_task && (int)(hoff[j] - col0) <= s) ++j;
                const int window_end = min((int)(hoff[j - 1] - col0) + 63, nsteps);
                if (s < window_end) {
#pragma unroll 1
                    for (; s < window_end; ++s) step(s, std::true_type{});
                    continue;
                }
                const int next_boundary = (j <= nh_task) ? (int)(hoff[j] - col0) : nsteps;
#pragma unroll 1
                for (; s < next_boundary; ++s) step(s, std::false_type{});
            }
            if (MULTI) __syncwarp();  // the next strip's lane 0 reads what this strip's lane 31 wrote
        }
    }
}

size_t pd_bucket_smem_bytes(int k) {
    return (size_t)(128 / 32) * (((k + 1) / 2) * kBases * 32 * sizeof(float4) + (size_t)k * 3 * 32 * sizeof(float2));
}

template <int K, bool MULTI>
int launch_pd_bucket_k(const DevTables &t, const DevBatch &b, const uint8_t *ops, int grid, cudaStream_t s) {
    const size_t smem = pd_bucket_smem_bytes(K);
    if (smem > 48 * 1024) {
        const cudaError_t e =
            cudaFuncSetAttribute(pd_bucket_kernel<K, MULTI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    pd_bucket_kernel<K, MULTI><<<grid, 128, smem, s>>>(t, b, ops);
    return (int)cudaGetLastError();
}

template <int K, bool MULTI>
int pd_bucket_occupancy_k(int *blocks_per_sm) {
    const void *fn = (const void *)pd_bucket_kernel<K, MULTI>;
    const size_t smem = pd_bucket_smem_bytes(K);
    if (smem > 48 * 1024) {  // (above 48 KB the kernel must opt in before the query counts it)
        const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return (int)e;
    }
    return (int)cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, fn, 128, smem);
}

}  // namespace

// key: rows per lane (2..8) in the low bits, 16 for multi-strip tasks, as the regular buckets
int launch_pd_bucket(const DevTables &t, const DevBatch &b, const uint8_t *ops, int key, int grid, cudaStream_t s) {
    const bool multi = (key & 16) != 0;
    switch (key & 15) {
#define GHMM_PD_BUCKET(KK)                                                  \
    case KK:                                                                \
        return multi ? launch_pd_bucket_k<KK, true>(t, b, ops, grid, s)     \
                     : launch_pd_bucket_k<KK, false>(t, b, ops, grid, s);
        GHMM_PD_BUCKET(2)
        GHMM_PD_BUCKET(3)
        GHMM_PD_BUCKET(4)
        GHMM_PD_BUCKET(5)
        GHMM_PD_BUCKET(6)
        GHMM_PD_BUCKET(7)
        GHMM_PD_BUCKET(8)
#undef GHMM_PD_BUCKET
        default: return (int)cudaErrorInvalidValue;
    }
}

int pd_bucket_occupancy(int key, int *blocks_per_sm) {
    const bool multi = (key & 16) != 0;
    switch (key & 15) {
#define GHMM_PD_OCC(KK) \
    case KK:            \
        return multi ? pd_bucket_occupancy_k<KK, true>(blocks_per_sm) : pd_bucket_occupancy_k<KK, false>(blocks_per_sm);
        GHMM_PD_OCC(2)
        GHMM_PD_OCC(3)
        GHMM_PD_OCC(4)
        GHMM_PD_OCC(5)
        GHMM_PD_OCC(6)
        GHMM_PD_OCC(7)
        GHMM_PD_OCC(8)
#undef GHMM_PD_OCC
        default: return (int)cudaErrorInvalidValue;
    }
}

}  // namespace ghmm
