// prep.cu -- read preparation before the PairHMM, on the device: what PairHMMLikelihoodCalculationEngine.
// modifyReadQualities does to each read on the host in GATK (src/main/java/org/broadinstitute/hellbender/tools/
// walkers/haplotypecaller/PairHMMLikelihoodCalculationEngine.java:283-322,331-371):
//   - the PCR indel error model: at every position but the last, insertion and deletion qualities are capped by the
//     model's quality for the tandem-repeat length there (findTandemRepeatUnits, ReadLikelihoodCalculationEngine.
//     java:193-253, repeat units up to 8 bases, lengths capped at 20);
//   - base qualities capped by the mapping quality (unless disabled), then base qualities below the threshold and
//     insertion / deletion qualities below 6 set to 6 (compared as Java's signed bytes).
// The batch's planes hold the raw values (missing insertion / deletion qualities as 45, the constant gap continuation
// penalty filled in); prep_kernel rewrites quals, ins and dels in place, one warp per read with its lanes over the
// positions.  With the DRAGstr imputation (DragstrPairHMMInputScoreImputator.java:54-88, DragstrReadSTRAnalyzer)
// dragstr_kernel caps the base qualities and writes ins, dels and gcp instead, also one warp per read.
#include <cuda_runtime.h>

#include <cstdint>

#include "ghmm_internal.h"

namespace ghmm {
namespace {

constexpr int kMaxUnit = 8;
constexpr int kMaxRepeat = 20;

// findNumberOfRepetitions over sub-ranges of the read: copies of unit b[u, u+L) at the start (leading) or the end
// (trailing) of b[t, t+n)
__device__ __forceinline__ int repetitions(const uint8_t *b, int u, int L, int t, int n, bool leading) {
    if (n == 0) return 0;
    int count = 0;
    if (leading) {
        for (int s = 0; s <= n - L; s += L) {
            for (int k = 0; k < L; ++k)
                if (b[t + s + k] != b[u + k]) return count;
            ++count;
        }
    } else {
        for (int s = n - L; s >= 0; s -= L) {
            for (int k = 0; k < L; ++k)
                if (b[t + s + k] != b[u + k]) return count;
            ++count;
        }
    }
    return count;
}

__device__ __forceinline__ bool same_unit(const uint8_t *b, int u1, int l1, int u2, int l2) {
    if (l1 != l2) return false;
    for (int k = 0; k < l1; ++k)
        if (b[u1 + k] != b[u2 + k]) return false;
    return true;
}

// findTandemRepeatUnits(...).getRight() at `offset` of a read of n bases
__device__ __forceinline__ int tandem_repeat_length(const uint8_t *b, int n, int offset) {
    int max_bw = 0, bw_u = offset, bw_l = 1;
    for (int L = 1; L <= kMaxUnit; ++L) {
        if (offset + 1 - L < 0) break;
        max_bw = repetitions(b, offset - L + 1, L, 0, offset + 1, false);
        if (max_bw > 1) {
            bw_u = offset - L + 1;
            bw_l = L;
            break;
        }
    }
    int max_rl = max_bw;
    if (offset < n - 1) {
        int fw_u = offset + 1, fw_l = 1, max_fw = 0;
        for (int L = 1; L <= kMaxUnit; ++L) {
            if (offset + L + 1 > n) break;
            max_fw = repetitions(b, offset + 1, L, offset + 1, n - offset - 1, true);
            if (max_fw > 1) {
                fw_l = L;
                break;
            }
        }
        if (same_unit(b, fw_u, fw_l, bw_u, bw_l))
            max_rl = max_bw + max_fw;
        else
            max_rl = max_fw + repetitions(b, fw_u, fw_l, 0, offset + 1, false);
    }
    return max_rl > kMaxRepeat ? kMaxRepeat : max_rl;
}

__device__ __forceinline__ int as_java_byte(int v) { return v > 127 ? v - 256 : v; }

// bases a warp stages in shared memory for the tandem-repeat search; longer reads are searched in place
constexpr int kPrepWarps = 8;
constexpr int kPrepStage = 1024;

__device__ __forceinline__ uint8_t cap_base_quality(int q, int mapq, const PrepArgs &P) {
    if (P.cap_to_mapq) q = (q < mapq ? q : mapq) & 0xFF;
    if (as_java_byte(q) < P.threshold) q = 6;
    return (uint8_t)q;
}

// v / p for 0 <= v < 2^17 and 2 <= p <= 32, with magic = ceil(2^32 / p); p = 1 passes v through
__device__ __forceinline__ int div_period(int v, int p, uint32_t magic) {
    return p == 1 ? v : (int)__umulhi((uint32_t)v, magic);
}

__device__ __forceinline__ uint32_t period_magic(int p) {
    return (uint32_t)((0x100000000ull + (uint64_t)p - 1) / (uint64_t)p);
}

// Where D[j] = (base j == base j + p) is 0, for the n bases of S (D is 0 from n - p on): ZM[c] is the zero mask of
// positions 32 c .. 32 c + 31 (one ballot each), PZ[c] the nearest zero before the chunk (-1 if none) and NZ[c] the
// nearest zero after it (n if none), found 32 chunks per ballot.  Together they answer "nearest zero at or after y"
// and "nearest zero before y" for any y in [0, n) in a few instructions.  Warp-collective; ends with __syncwarp.
__device__ __forceinline__ void zero_index(const uint8_t *S, int n, int p, uint32_t *ZM, uint32_t *PZ, uint32_t *NZ,
                                           int lane) {
    const int nch = (n + 31) >> 5;
    for (int c = 0; c < nch; ++c) {
        const int x = (c << 5) + lane;
        const bool d = x + p < n && S[x] == S[x + p];
        const uint32_t z = __ballot_sync(0xffffffffu, !d);
        if (lane == 0) ZM[c] = z;
    }
    __syncwarp();
    int carry = -1;  // lane j of a group handles chunk 32 g + j
    for (int g = 0; g < nch; g += 32) {
        const int c = g + lane;
        const uint32_t zm = c < nch ? ZM[c] : 0u;
        const uint32_t has = __ballot_sync(0xffffffffu, zm != 0u);
        const uint32_t below = has & ((1u << lane) - 1u);
        const int kb = below ? 31 - __clz(below) : 0;
        const uint32_t zb = __shfl_sync(0xffffffffu, zm, kb);
        if (c < nch) PZ[c] = (uint32_t)(below ? ((g + kb) << 5) + 31 - __clz(zb) : carry);
        if (has) {
            const int kl = 31 - __clz(has);
            carry = ((g + kl) << 5) + 31 - __clz(__shfl_sync(0xffffffffu, zm, kl));
        }
    }
    carry = n;
    for (int g = (nch - 1) & ~31; g >= 0; g -= 32) {
        const int c = g + lane;
        const uint32_t zm = c < nch ? ZM[c] : 0u;
        const uint32_t has = __ballot_sync(0xffffffffu, zm != 0u);
        const uint32_t above = lane < 31 ? has >> (lane + 1) : 0u;
        const int ka = above ? lane + __ffs(above) : 0;
        const uint32_t za = __shfl_sync(0xffffffffu, zm, ka);
        if (c < nch) NZ[c] = (uint32_t)(above ? ((g + ka) << 5) + __ffs(za) - 1 : carry);
        if (has) {
            const int kf = __ffs(has) - 1;
            carry = ((g + kf) << 5) + __ffs(__shfl_sync(0xffffffffu, zm, kf)) - 1;
        }
    }
    __syncwarp();
}

__device__ __forceinline__ int zero_at_or_after(const uint32_t *ZM, const uint32_t *NZ, int y) {
    const uint32_t a = ZM[y >> 5] >> (y & 31);
    return a ? y + __ffs(a) - 1 : (int)NZ[y >> 5];
}

__device__ __forceinline__ int zero_before(const uint32_t *ZM, const uint32_t *PZ, int y) {
    const uint32_t b = ZM[y >> 5] & ((1u << (y & 31)) - 1u);
    return b ? ((y >> 5) << 5) + 31 - __clz(b) : (int)PZ[y >> 5];
}

// findTandemRepeatUnits(bases, offset).getRight() for every offset of a staged read, from the runs of D for unit
// lengths L = 1..8.  A unit of L bases ending at offset repeats 1 + floor(run of ones of D ending at offset - L / L)
// times backward; the unit after offset repeats 1 + floor(run of ones starting at offset + 1 / L) times forward;
// the first L with more than one copy is the unit, as in the Java loops.  The units are equal when both loops stop
// at the same L and D is 1 over [offset - L + 1, offset]; otherwise the forward unit's copies ending at offset are
// floor(run of ones ending at offset / L).  Per offset the state of the two loops packs into one word:
// bits 0-3 backward L (0: not found), 4-8 its copies, 9-12 forward L, 13-17 its copies, 18-22 copies of the forward
// unit ending at offset, 23 D1[offset], 24-28 the run of D1 ones ending at offset, 29 units equal.  Copies are
// capped at 21, which keeps min(sum, 20) exact.
__device__ __forceinline__ int cap21(int v) { return v < 21 ? v : 21; }

__device__ __forceinline__ void tandem_pass(const uint32_t *ZM, const uint32_t *PZ, const uint32_t *NZ, uint32_t *st,
                                            int n, int L, uint32_t magic, int lane) {
    for (int off = lane; off < n - 1; off += 32) {
        uint32_t w = st[off];
        if (L == 1) w = 0;
        int bwL = w & 15, fwL = (w >> 9) & 15;
        if (bwL == 0 && off + 1 - L >= 0) {
            const int s = off + 1 - L;
            const int c = 1 + div_period(s - 1 - zero_before(ZM, PZ, s), L, magic);
            if (c > 1) {
                bwL = L;
                w |= (uint32_t)L | ((uint32_t)cap21(c) << 4);
            }
        }
        if (fwL == 0 && off + L + 1 <= n) {
            const int x = off + 1;
            const int c = 1 + div_period(zero_at_or_after(ZM, NZ, x) - x, L, magic);
            if (c > 1) {
                fwL = L;
                const int rep = div_period(x - 1 - zero_before(ZM, PZ, x), L, magic);
                w |= ((uint32_t)L << 9) | ((uint32_t)cap21(c) << 13) | ((uint32_t)cap21(rep) << 18);
            }
        }
        if (L == 1) {
            const uint32_t d1 = zero_at_or_after(ZM, NZ, off) > off ? 1u : 0u;
            w |= (d1 << 23) | ((uint32_t)cap21(off - zero_before(ZM, PZ, off + 1)) << 24);
        }
        if (bwL == L && fwL == L && zero_at_or_after(ZM, NZ, off - L + 1) >= off + 1) w |= 1u << 29;
        st[off] = w;
    }
}

__device__ __forceinline__ int tandem_from_state(uint32_t w) {
    const int bwL = w & 15, fwL = (w >> 9) & 15;
    const int bw = bwL ? (int)((w >> 4) & 31) : 1, fw = fwL ? (int)((w >> 13) & 31) : 1;
    const int lb = bwL ? bwL : 1, lf = fwL ? fwL : 1;
    const bool same = lb == lf && (lb == 1 ? ((w >> 23) & 1u) : ((w >> 29) & 1u));
    const int rep = fwL ? (int)((w >> 18) & 31) : (int)((w >> 24) & 31);
    const int rl = same ? bw + fw : fw + rep;
    return rl < kMaxRepeat ? rl : kMaxRepeat;
}

__global__ void prep_kernel(DevBatch B, uint8_t *quals, uint8_t *ins, uint8_t *dels, int64_t n_reads, PrepArgs P) {
    __shared__ uint8_t stage[kPrepWarps][kPrepStage];
    __shared__ uint32_t state[kPrepWarps][kPrepStage];
    __shared__ uint32_t zidx[kPrepWarps][3 * (kPrepStage / 32)];
    __shared__ uint8_t cache[24];  // indexed by repeat length: shared rather than a local copy of the parameter
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
#pragma unroll
        for (int k = 0; k < 24; ++k) cache[k] = P.pcr_cache[k];
    }
    __syncthreads();
    uint32_t *ZM = zidx[w], *PZ = ZM + kPrepStage / 32, *NZ = PZ + kPrepStage / 32;
    for (int64_t r = (int64_t)blockIdx.x * kPrepWarps + w; r < n_reads; r += (int64_t)gridDim.x * kPrepWarps) {
        const int64_t o = B.read_off[r];
        const int n = (int)(B.read_off[r + 1] - o);
        const bool staged = P.pcr && n > 1 && n <= kPrepStage;
        if (staged) {
            for (int x = lane; x < n; x += 32) stage[w][x] = B.bases[o + x];
            __syncwarp();
            const int top = n - 1 < kMaxUnit ? n - 1 : kMaxUnit;
            for (int L = 1; L <= top; ++L) {
                zero_index(stage[w], n, L, ZM, PZ, NZ, lane);
                tandem_pass(ZM, PZ, NZ, state[w], n, L, period_magic(L), lane);
                __syncwarp();
            }
        }
        const int mapq = P.mapq[r];
        for (int x = lane; x < n; x += 32) {
            quals[o + x] = cap_base_quality(quals[o + x], mapq, P);
            int iq = ins[o + x], dq = dels[o + x];
            if (P.pcr && x < n - 1) {  // applyPCRErrorModel: min as unsigned bytes
                const int rl = staged ? tandem_from_state(state[w][x]) : tandem_repeat_length(B.bases + o, n, x);
                const int cap = cache[rl];
                iq = iq < cap ? iq : cap;
                dq = dq < cap ? dq : cap;
            }
            ins[o + x] = (uint8_t)(as_java_byte(iq) < 6 ? 6 : iq);
            dels[o + x] = (uint8_t)(as_java_byte(dq) < 6 ? 6 : dq);
        }
        __syncwarp();
    }
}

// Java's Math.round(double) (half up), cast to a byte
__device__ __forceinline__ uint8_t java_round_byte(double x) {
    double r = floor(x);
    if (x - r >= 0.5) r += 1.0;
    return (uint8_t)((long long)r & 0xFF);
}

// DRAGstr imputation, one warp per read, in shared memory.  DragstrReadSTRAnalyzer's repeat count of period p at
// position i is the longest tandem run, in units of p, of a p-mer starting at x in [i - p + 1, i + 1] (a unit
// starting at 0 counts one repeat fewer, not below 1, for positions before p - 1); the most repeated period wins,
// ties to the shorter one.  The run through the unit at x is 1 + F + Bk copies, where F copies follow it and Bk
// precede it.  With D[j] = (base j == base j + p), the units at x and x + p are equal exactly when D is 1 over
// [x, x + p), so F = floor(LF / p) for LF the run of ones of D starting at x, and Bk = floor(LB / p) for LB the run
// of ones ending at x - 1: both follow from the nearest zeros of D on either side of x.  Per period: the zero masks
// of D, 32 positions per ballot; the nearest zero before and after every 32-position chunk, 32 chunks per ballot;
// the counts of every unit start; the maximum over every position's window of p + 1 unit starts.
struct StrWarp {  // one warp's shared memory for a read of up to lpad - 1 bases
    uint8_t *S;              // bases
    uint32_t *ZM, *PZ, *NZ;  // per chunk: zero mask of D, nearest zero before it, nearest zero at or after its end
    int16_t *C;              // run count of the unit starting at x (0 past the last unit start, as window padding)
    int16_t *BR;             // most repeats so far
    uint8_t *BP;             // their period
};

// one period of the analysis, called from one place with the period at run time: a single copy of the code keeps
// the kernel small enough for the instruction cache
__device__ __forceinline__ void str_period(const StrWarp &W, int p, int n, int lane) {
    const uint32_t magic = period_magic(p);
    const int nu = n - p + 1;  // unit starts 0 .. n - p
    const int nch = (n + 31) >> 5;
    zero_index(W.S, n, p, W.ZM, W.PZ, W.NZ, lane);
    for (int c = 0; c < nch; ++c) {
        const int x = (c << 5) + lane;
        const uint32_t z = W.ZM[c];
        const uint32_t ahead = z >> lane, behind = z & ((1u << lane) - 1u);
        const int nz = ahead ? x + __ffs(ahead) - 1 : (int)W.NZ[c];
        const int pz = behind ? (c << 5) + 31 - __clz(behind) : (int)W.PZ[c];
        if (x < nu) W.C[x] = (int16_t)(1 + div_period(nz - x, p, magic) + div_period(x - 1 - pz, p, magic));
        else if (x <= n) W.C[x] = 0;
    }
    if (lane == 0 && (n & 31) == 0) W.C[n] = 0;
    __syncwarp();
    for (int i = lane; i < n; i += 32) {
        int best = 0;
        if (i >= p - 1) {
            const int16_t *w = W.C + (i - p + 1);
            for (int k = 0; k <= p; ++k) best = max(best, (int)w[k]);
        } else {  // the window starts at the read's first base, whose unit counts one repeat fewer here
            best = max(W.C[0] - 1, 1);
            for (int x = 1; x <= i + 1; ++x) best = max(best, (int)W.C[x]);
        }
        if (p == 1 || best > W.BR[i]) {
            W.BR[i] = (int16_t)best;
            W.BP[i] = (uint8_t)p;
        }
    }
    __syncwarp();
}

// 6 blocks of 8 warps per SM: 40 registers a thread
__global__ void __launch_bounds__(256, 6) dragstr_kernel(DevBatch B, uint8_t *quals, uint8_t *ins, uint8_t *dels,
                                                         uint8_t *gcp, int64_t n_reads, PrepArgs P, int lpad,
                                                         int wstride) {
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, wpb = blockDim.x >> 5;
    unsigned char *base = smem + (size_t)w * wstride;
    const int nchunk = lpad >> 5;
    StrWarp W;
    W.S = base;
    W.ZM = reinterpret_cast<uint32_t *>(base + lpad);
    W.PZ = W.ZM + nchunk;
    W.NZ = W.PZ + nchunk;
    W.C = reinterpret_cast<int16_t *>(W.NZ + nchunk);
    W.BR = W.C + lpad;
    W.BP = reinterpret_cast<uint8_t *>(W.BR + lpad);
    const int maxp = P.str_max_period, maxr = P.str_max_repeats;
    for (int64_t r = (int64_t)blockIdx.x * wpb + w; r < n_reads; r += (int64_t)gridDim.x * wpb) {
        const int64_t o = B.read_off[r];
        const int n = (int)(B.read_off[r + 1] - o);
        const int mapq = P.mapq[r];
        for (int x = lane; x < n; x += 32) {
            W.S[x] = B.bases[o + x];
            quals[o + x] = cap_base_quality(quals[o + x], mapq, P);
        }
        __syncwarp();
        const int top = maxp < n ? maxp : n;
        for (int p = 1; p <= top; ++p) str_period(W, p, n, lane);
        // DragstrPairHMMInputScoreImputator.impute with DragstrParams.lookup's clamping of period and repeats
        for (int i = lane; i < n - 1; i += 32) {
            const int per = W.BP[i], rep = W.BR[i];
            const int pi = per < maxp ? per - 1 : maxp - 1, ri = rep < maxr ? rep - 1 : maxr - 1;
            const double g = P.str_gop[pi * maxr + ri], c = P.str_gcp[pi * maxr + ri];
            const uint8_t gb = java_round_byte(g < 40.0 ? g : 40.0);
            ins[o + i] = gb;
            dels[o + i] = gb;
            gcp[o + i] = java_round_byte(c);
        }
        if (lane == 0 && n > 0) {
            ins[o + n - 1] = 45;
            dels[o + n - 1] = 45;
            gcp[o + n - 1] = 10;
        }
        __syncwarp();
    }
}

}  // namespace

int launch_dragstr(const DevBatch &b, int64_t n_reads, const PrepArgs &p, int sm_count, cudaStream_t s) {
    if (n_reads <= 0) return 0;
    const int lpad = (p.max_read_len + 1 + 31) / 32 * 32;  // one spare base: the count array is read up to n
    // bases, C and best repeats (16-bit), best periods, and three 32-bit words per 32 bases
    const size_t per_warp = ((size_t)lpad * 6 + (size_t)(lpad / 32) * 12 + 15) / 16 * 16;
    int wpb = (int)(32768 / per_warp);
    wpb = wpb < 1 ? 1 : wpb > 8 ? 8 : wpb;
    const size_t smem = per_warp * wpb;
    if (smem > 49152) {
        cudaError_t e = cudaFuncSetAttribute(dragstr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e) return (int)e;
    }
    const int64_t want = (n_reads + wpb - 1) / wpb;
    const int64_t cap = (int64_t)sm_count * (48 / wpb);  // the blocks that are resident at once
    const int grid = (int)(want < cap ? want : cap);
    dragstr_kernel<<<grid, 32 * wpb, smem, s>>>(b, const_cast<uint8_t *>(b.quals), const_cast<uint8_t *>(b.ins),
                                              const_cast<uint8_t *>(b.dels), const_cast<uint8_t *>(b.gcp), n_reads, p,
                                              lpad, (int)per_warp);
    return (int)cudaGetLastError();
}

int launch_prep(const DevBatch &b, int64_t n_reads, const PrepArgs &p, int sm_count, cudaStream_t s) {
    if (n_reads <= 0) return 0;
    const int64_t want = (n_reads + kPrepWarps - 1) / kPrepWarps;
    const int64_t cap = (int64_t)sm_count * 8;
    const int grid = (int)(want < cap ? want : cap);
    // the planes are the batch's own device buffers (DevBatch holds them as const for the forward kernels)
    prep_kernel<<<grid, kPrepWarps * 32, 0, s>>>(b, const_cast<uint8_t *>(b.quals), const_cast<uint8_t *>(b.ins),
                                                 const_cast<uint8_t *>(b.dels), n_reads, p);
    return (int)cudaGetLastError();
}

}  // namespace ghmm
