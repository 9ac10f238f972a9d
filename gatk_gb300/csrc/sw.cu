// sw.cu -- Smith-Waterman alignment on the device: what GATK's SmithWatermanJavaAligner computes
// (src/main/java/org/broadinstitute/hellbender/utils/smithwaterman/SmithWatermanJavaAligner.java:59-379) and what the
// native SWAlignerNativeBinding.align returns (SWNativeAlignerWrapper.java:31-59): a cigar and an alignment offset
// of `alt` against `ref`, for the four overhang strategies, bit-identical to the Java code.
//
// Pipeline of one batch (all on one stream):
//   sw_forward_kernel<K>  one warp per alignment.  The exact-substring shortcut (Utils.lastIndexOf, Utils.java:
//                         1124-1138) is tested first when enabled.  Otherwise an anti-diagonal wavefront fills the
//                         score recurrence of calculateMatrix (:109-228): lane l owns K consecutive alt columns,
//                         the warp streams over the ref rows, each lane passing its last column's score and the
//                         row's best horizontal gap to the next lane every step.  Alts longer than 32*K run in
//                         strips of 32*K columns whose boundary column goes through a per-pair scratch.  Per cell
//                         it keeps 4 traceback bits (not diagonal; horizontal >= vertical; vertical gap opened here;
//                         horizontal gap opened here), from which the traceback rebuilds the backtrack entry
//                         0 / -ki / +kd exactly: a gap's length is the distance to the cell that opened it.  The last
//                         column's and the bottom row's scores go to an edge array for the end-cell choice.
//   sw_traceback_kernel   one thread per alignment: end cell per strategy, traceback, cigar elements in reverse
//                         into a per-pair slot (calculateCigar, :261-379).
//   sw_scan_kernel        exclusive prefix sums (one block) of per-pair counts.
//   sw_gather_kernel      slot -> compact, forward-ordered BAM-encoded cigar ops.
// Scores are int32 with Java's wrapping adds; every comparison is the Java one, so ties resolve identically.
#include <cuda_runtime.h>

#include <cstdint>

#include "ghmm_internal.h"

namespace ghmm {
namespace {

constexpr int kSwCutoff = -100000000;       // MATRIX_MIN_CUTOFF (int) -1.0e8
constexpr int kSwLowInit = INT32_MIN / 2;   // lowInitValue = Integer.MIN_VALUE / 2

__device__ __forceinline__ int wadd(int a, int b) { return (int)((unsigned)a + (unsigned)b); }
__device__ __forceinline__ int wsub(int a, int b) { return (int)((unsigned)a - (unsigned)b); }

// top row / left column of the score matrix: 0, or gap open + (k - 1) gap extends for INDEL and LEADING_INDEL
__device__ __forceinline__ int edge_init(const SwArgs &A, int64_t k) {
    if (!A.indel_edges || k <= 0) return 0;
    return (int)((unsigned)A.open + (unsigned)(k - 1) * (unsigned)A.extend);
}

// Utils.lastIndexOf by one warp: the largest r with ref[r, r+m) == alt, or -1
__device__ int warp_last_index_of(const uint8_t *ref, int n, const uint8_t *alt, int m) {
    const int lane = threadIdx.x & 31;
    for (int base = n - m; base >= 0; base -= 32) {
        const int r = base - lane;
        bool hit = false;
        if (r >= 0) {
            int q = 0;
            while (q < m && ref[r + q] == alt[q]) ++q;
            hit = q == m;
        }
        const unsigned b = __ballot_sync(0xffffffffu, hit);
        if (b) return base - (__ffs(b) - 1);
    }
    return -1;
}

// bits |= mask when a > b (a >= b): one compare and one predicated OR
__device__ __forceinline__ void or_if_gt(uint32_t &bits, int a, int b, uint32_t mask) {
    asm("{\n\t.reg .pred p;\n\tsetp.gt.s32 p, %1, %2;\n\t@p or.b32 %0, %0, %3;\n\t}"
        : "+r"(bits)
        : "r"(a), "r"(b), "r"(mask));
}
__device__ __forceinline__ void or_if_ge(uint32_t &bits, int a, int b, uint32_t mask) {
    asm("{\n\t.reg .pred p;\n\tsetp.ge.s32 p, %1, %2;\n\t@p or.b32 %0, %0, %3;\n\t}"
        : "+r"(bits)
        : "r"(a), "r"(b), "r"(mask));
}

// What one lane needs across the steps of a strip.
struct StripCtx {
    const uint8_t *ref;
    uint32_t *tb;          // this lane's traceback word of step 0 (words of a step are 32 apart)
    int *lastrow;          // the lane holding the alt's last column: its K scores + open per row (kSwRowStride ints)
    const int2 *strip_in;  // lane 0 after the first strip: (score, horizontal gap) of the previous strip's last column
    int2 *strip_out;       // lane 31 before the last strip
    int n, open, ext;
    int match_o, mismatch_o;  // match / mismatch minus the gap open penalty (scores are carried as H + open)
    bool inject;           // lane 0 of the first strip: the matrix's left edge
    bool indel_edges;
    bool owns_last;
};

template <int K>
struct LaneState {
    uint8_t b[K];   // alt bases of the lane's columns
    int hup[K];     // H[i-1][j] + open before a step, H[i][j] + open after it
    int bv[K];      // best vertical gap of each column
    int hdiag;      // H[i-1][first column - 1] + open
    int send_h, send_b;
    uint8_t a_next;
};

// One anti-diagonal step of one lane: row i = t - lane + 1 over the lane's K columns.  CHECK: some lanes of the
// warp are outside the matrix this step (the first and last 31 steps of a strip).  Scores travel as H + open: the
// one add per cell then serves as the next row's vertical gap opening and the next column's horizontal one, and
// the diagonal adds the score minus open.  Every sum is the Java one modulo 2^32.
template <int K, bool CLAMP, bool CHECK>
__device__ __forceinline__ void sw_step(const StripCtx &C, LaneState<K> &L, int t, int lane) {
    const int i = t - lane + 1;
    const bool active = !CHECK || (i >= 1 && i <= C.n);
    const uint8_t a = L.a_next;
    L.a_next = C.ref[min(max(i, 0), C.n - 1)];  // the next step's row is i + 1, whose base is ref[i]
    int h_left = __shfl_up_sync(0xffffffffu, L.send_h, 1);
    int bh = __shfl_up_sync(0xffffffffu, L.send_b, 1);
    if (lane == 0) {
        if (C.inject) {
            h_left = wadd(C.indel_edges && i > 0 ? (int)((unsigned)C.open + (unsigned)(i - 1) * (unsigned)C.ext) : 0,
                          C.open);
            bh = kSwLowInit;
        } else if (active) {
            const int2 v = C.strip_in[i];
            h_left = v.x;
            bh = v.y;
        }
    }
    if (!active) return;
    uint32_t bits = 0;
    int hd = L.hdiag;
    int hl = h_left;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int diag = wadd(hd, a == L.b[k] ? C.match_o : C.mismatch_o);
        const int bvk = wadd(L.bv[k], C.ext), pv = L.hup[k];
        const int v = max(bvk, pv);
        const int bhk = wadd(bh, C.ext), ph = hl;
        const int h = max(bhk, ph);
        const int g = max(h, v);
        int hn = max(diag, g);
        if (CLAMP) hn = max(hn, kSwCutoff);
        or_if_gt(bits, g, diag, 1u << (4 * k));  // not diagonal: diag < max(right, down)
        or_if_ge(bits, h, v, 2u << (4 * k));     // right >= down
        or_if_gt(bits, pv, bvk, 4u << (4 * k));  // vertical gap opened here
        or_if_gt(bits, ph, bhk, 8u << (4 * k));  // horizontal gap opened here
        const int hno = wadd(hn, C.open);
        L.bv[k] = v;
        bh = h;
        hd = L.hup[k];
        L.hup[k] = hno;
        hl = hno;
    }
    C.tb[(int64_t)t * 32] = bits;
    if (C.owns_last) {
        int4 *row = reinterpret_cast<int4 *>(C.lastrow + (int64_t)(i - 1) * kSwRowStride(K));
#pragma unroll
        for (int q = 0; q < K; q += 4)
            row[q / 4] = make_int4(L.hup[q], q + 1 < K ? L.hup[q + 1 < K ? q + 1 : 0] : 0,
                                   q + 2 < K ? L.hup[q + 2 < K ? q + 2 : 0] : 0,
                                   q + 3 < K ? L.hup[q + 3 < K ? q + 3 : 0] : 0);
    }
    if (C.strip_out && lane == 31) C.strip_out[i] = make_int2(hl, bh);
    L.send_h = hl;
    L.send_b = bh;
    L.hdiag = h_left;
}

template <int K, bool CLAMP>
__device__ __forceinline__ void sw_strip(const SwArgs &A, const SwPair &P, int s, int nstrips) {
    const int lane = threadIdx.x & 31;
    const int n = P.ref_len, m = P.alt_len;
    const int col0 = s * 32 * K;               // alt columns of this strip: col0+1 .. col0+32K (1-based)
    const int jbase = col0 + lane * K;         // this lane's columns: jbase+1 .. jbase+K
    const uint8_t *alt = A.alt_plane + P.alt_off;
    const bool last_strip = s == nstrips - 1;
    StripCtx C;
    C.ref = A.ref_plane + P.ref_off;
    C.n = n;
    C.open = A.open;
    C.ext = A.extend;
    C.match_o = wsub(A.match, A.open);
    C.mismatch_o = wsub(A.mismatch, A.open);
    C.inject = s == 0;
    C.indel_edges = A.indel_edges != 0;
    const int km = (m - 1) - jbase;            // the alt's last column, on its lane in the last strip
    C.owns_last = last_strip && km >= 0 && km < K;
    const int64_t steps = (int64_t)n + 31;
    C.tb = A.tb + P.tb_off + (int64_t)s * steps * 32 + lane;
    C.lastrow = A.edges + P.edge_off;
    C.strip_in = s > 0 ? A.strip_scratch + P.scratch_off : nullptr;
    C.strip_out = !last_strip ? A.strip_scratch + P.scratch_off : nullptr;
    LaneState<K> L;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int j = jbase + k + 1;
        L.b[k] = j <= m ? alt[j - 1] : 0;
        L.hup[k] = wadd(edge_init(A, j), A.open);
        L.bv[k] = kSwLowInit;
    }
    L.hdiag = wadd(edge_init(A, jbase), A.open);  // H[0][jbase] + open
    L.send_h = 0;
    L.send_b = kSwLowInit;
    L.a_next = C.ref[min(max(0 - lane, 0), n - 1)];
    int t = 0;
    for (; t < 31; ++t) sw_step<K, CLAMP, true>(C, L, t, lane);
#pragma unroll 4
    for (; t < n; ++t) sw_step<K, CLAMP, false>(C, L, t, lane);  // every lane inside the matrix
    for (; t < n + 31; ++t) sw_step<K, CLAMP, true>(C, L, t, lane);
    // the lanes finish on row n: their scores are the bottom row
    int *bottom = A.edges + P.edge_off + (int64_t)n * kSwRowStride(K);  // H[n][j] + open at bottom[j-1]
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int j = jbase + k + 1;
        if (j <= m) bottom[j - 1] = L.hup[k];
    }
    __syncwarp();
}

template <int K, bool CLAMP>
__global__ void __launch_bounds__(128) sw_forward_kernel(SwArgs A, const int32_t *tasks, int n_tasks, int *cursor) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int task = 0;
        if (lane == 0) task = atomicAdd(cursor, 1);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= n_tasks) break;
        const int p = tasks[task];
        const SwPair P = A.pairs[p];
        if (A.shortcut) {
            const int idx = warp_last_index_of(A.ref_plane + P.ref_off, P.ref_len, A.alt_plane + P.alt_off,
                                               P.alt_len);
            if (idx >= 0) {
                if (lane == 0) {
                    A.state[p] = 1;
                    A.offset[p] = idx;
                }
                continue;
            }
        }
        if (lane == 0) A.state[p] = 0;
        const int nstrips = (P.alt_len + 32 * K - 1) / (32 * K);
        for (int s = 0; s < nstrips; ++s) sw_strip<K, CLAMP>(A, P, s, nstrips);
    }
}

// traceback bits of cell (i, j), 1-based
__device__ __forceinline__ uint32_t tb_code(const SwArgs &A, const SwPair &P, int K, int i, int j) {
    const int w = 32 * K;
    const int s = (j - 1) / w, within = (j - 1) - s * w;
    const int lane = within / K, k = within - lane * K;
    const int64_t steps = (int64_t)P.ref_len + 31;
    const int64_t t = (int64_t)(i - 1) + lane;
    return (A.tb[P.tb_off + ((int64_t)s * steps + t) * 32 + lane] >> (4 * k)) & 15u;
}

__global__ void sw_traceback_kernel(SwArgs A, int n_pairs) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pairs) return;
    const SwPair P = A.pairs[p];
    const int n = P.ref_len, m = P.alt_len;
    uint32_t *slot = A.slot + P.slot_off;
    const int cap = 2 * m + 4;
    if (n <= 0) {           // a read whose region has no haplotype: not aligned
        A.n_ops[p] = 0;
        A.offset[p] = -1;
        return;
    }
    if (A.state[p] == 1) {  // exact-substring shortcut: cigar mM, offset already written
        slot[0] = ((uint32_t)m << 4) | kSwOpM;
        A.n_ops[p] = 1;
        return;
    }
    const int K = P.k;
    const int stride = kSwRowStride(K);
    const int km = (m - 1) % (32 * K) % K;  // the last column's place among its lane's columns
    const int *lastcol = A.edges + P.edge_off + km, *bottom = A.edges + P.edge_off + (int64_t)n * stride;
    int p1 = 0, p2 = 0;
    int maxscore = INT32_MIN;
    int segment = 0;
    if (A.strategy == kSwIndel) {
        p1 = n;
        p2 = m;
    } else {
        p2 = m;
        for (int i = 1; i <= n; ++i) {
            const int sc = wsub(lastcol[(int64_t)(i - 1) * stride], A.open);  // stored as H + open
            if (sc >= maxscore) {
                p1 = i;
                maxscore = sc;
            }
        }
        if (A.strategy != kSwLeadingIndel) {
            for (int j = 1; j <= m; ++j) {
                const int sc = wsub(bottom[j - 1], A.open);
                const int dn = n - j < 0 ? j - n : n - j, dc = p1 - p2 < 0 ? p2 - p1 : p1 - p2;
                if (sc > maxscore || (sc == maxscore && dn < dc)) {
                    p1 = n;
                    p2 = j;
                    maxscore = sc;
                    segment = m - j;
                }
            }
        }
    }
    int count = 0;
    bool overflow = false;
    auto push = [&](int op, int len) {
        if (count < cap)
            slot[count] = ((uint32_t)len << 4) | (uint32_t)op;
        else
            overflow = true;
        ++count;
    };
    if (segment > 0 && A.strategy == kSwSoftclip) {
        push(kSwOpS, segment);
        segment = 0;
    }
    int state = kSwOpM;
    int guard = n + m + 2;
    do {
        const uint32_t c = tb_code(A, P, K, p1, p2);
        int ns, step = 1;
        if (!(c & 1u)) {
            ns = kSwOpM;
        } else if (c & 2u) {  // horizontal: the gap's length is the distance back to the cell that opened it
            ns = kSwOpI;
            int q = p2;
            while (q > 1 && !(tb_code(A, P, K, p1, q) & 8u)) --q;
            step = p2 - q + 1;
        } else {              // vertical
            ns = kSwOpD;
            int r = p1;
            while (r > 1 && !(tb_code(A, P, K, r, p2) & 4u)) --r;
            step = p1 - r + 1;
        }
        if (ns == kSwOpM) {
            --p1;
            --p2;
        } else if (ns == kSwOpI) {
            p2 -= step;
        } else {
            p1 -= step;
        }
        if (ns == state) {
            segment += step;
        } else {
            if (segment > 0) push(state, segment);
            segment = step;
            state = ns;
        }
    } while (p1 > 0 && p2 > 0 && --guard > 0);
    int off;
    if (A.strategy == kSwSoftclip) {
        push(state, segment);
        if (p2 > 0) push(kSwOpS, p2);
        off = p1;
    } else if (A.strategy == kSwIgnore) {
        push(state, segment + p2);
        off = p1 - p2;
    } else {
        push(state, segment);
        if (p1 > 0)
            push(kSwOpD, p1);
        else if (p2 > 0)
            push(kSwOpI, p2);
        off = 0;
    }
    if (overflow || guard <= 0) {
        atomicExch(A.error, 1);
        count = 0;
    }
    A.n_ops[p] = count;
    A.offset[p] = off;
}

// exclusive prefix sums of `n` int32 counts into int64, starting at *running, which then advances by their sum
// (one block of 1024 threads, each over a contiguous chunk)
__global__ void __launch_bounds__(1024) sw_scan_kernel(const int32_t *counts, int64_t *starts, int64_t n,
                                                       int64_t *running) {
    __shared__ int64_t part[1024];
    const int t = threadIdx.x;
    const int64_t chunk = (n + 1023) / 1024;
    const int64_t b = min(n, (int64_t)t * chunk), e = min(n, b + chunk);
    int64_t sum = 0;
    for (int64_t i = b; i < e; ++i) sum += counts[i];
    part[t] = sum;
    __syncthreads();
    for (int d = 1; d < 1024; d <<= 1) {
        const int64_t v = t >= d ? part[t - d] : 0;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    const int64_t base = *running;
    int64_t run = base + part[t] - sum;
    for (int64_t i = b; i < e; ++i) {
        starts[i] = run;
        run += counts[i];
    }
    __syncthreads();
    if (t == 1023) *running = base + part[1023];
}

// reversed per-pair slots -> compact forward-ordered ops (an output that would pass ops_cap sets the error flag)
__global__ void sw_gather_kernel(SwArgs A, const int64_t *starts, uint32_t *ops, int64_t ops_cap, int n_pairs) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pairs) return;
    const int c = A.n_ops[p];
    if (starts[p] + c > ops_cap) {
        atomicExch(A.error, 2);
        return;
    }
    const uint32_t *slot = A.slot + A.pairs[p].slot_off;
    uint32_t *o = ops + starts[p];
    for (int q = 0; q < c; ++q) o[q] = slot[c - 1 - q];
}

constexpr double kInformativeThreshold = 0.2;  // AlleleLikelihoods.LOG_10_INFORMATIVE_THRESHOLD

// AlleleLikelihoods.searchBestAllele(sample, read, canBeReference = true, priorities) (AlleleLikelihoods.java:
// 505-560) over the read's row of the batch's likelihoods, and BestAllele.isInformative (:1269-1282)
__global__ void sw_realign_setup_kernel(DevBatch B, SwRealignArgs A) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < A.n_reads;
         r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t read = A.first_read + r;
        const int g = B.read_region[read];
        const int64_t h0 = B.region_hap_off[g];
        const int nh = (int)(B.region_hap_off[g + 1] - h0);
        if (nh <= 0) {
            A.best[read] = -1;
            A.informative[read] = 0;
            continue;
        }
        const double *row = B.out + B.out_off[g] + (read - B.region_read_off[g]) * nh;
        int best = 0, second = 0;
        double best_l = row[0], second_l = -INFINITY;
        for (int a = 1; a < nh; ++a) {
            const double c = row[a];
            if (c > best_l) {
                second = best;
                best = a;
                second_l = best_l;
                best_l = c;
            } else if (c > second_l) {
                second = a;
                second_l = c;
            }
        }
        if (A.priority && __dsub_rn(best_l, second_l) < kInformativeThreshold) {
            const double *prio = A.priority + h0;
            double best_p = prio[best], second_p = prio[second];
            for (int a = 0; a < nh; ++a) {
                const double c = row[a];
                if (a == best || __dsub_rn(best_l, c) > kInformativeThreshold) continue;
                const double cp = prio[a];
                if (cp > best_p) {
                    second = best;
                    best = a;
                    second_p = best_p;
                    best_p = cp;
                } else if (cp > second_p) {
                    second = a;
                    second_p = cp;
                }
            }
        }
        best_l = row[best];
        second_l = second != best ? row[second] : -INFINITY;
        const double confidence = best_l == second_l ? 0.0 : __dsub_rn(best_l, second_l);
        A.best[read] = best;
        A.informative[read] = confidence > kInformativeThreshold ? 1 : 0;
        SwPair &P = A.pairs[read];
        const int64_t h = h0 + best;
        P.ref_off = B.hap_off[h];
        P.ref_len = (int)(B.hap_off[h + 1] - B.hap_off[h]);
    }
}

// Peak of the int32 max/compare pipe the score recurrence leans on: eight independent chains of max.s32 per
// thread, written as PTX so the compiler keeps every one.
__global__ void __launch_bounds__(256) int32_max_peak_kernel(int *out, int iters, int seed) {
    int a0 = threadIdx.x ^ seed, a1 = a0 + 1, a2 = a0 + 2, a3 = a0 + 3, a4 = a0 + 4, a5 = a0 + 5, a6 = a0 + 6,
        a7 = a0 + 7;
    const int b0 = seed ^ blockIdx.x, b1 = b0 - 3;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            asm volatile("max.s32 %0, %0, %1;" : "+r"(a0) : "r"(b0));
            asm volatile("max.s32 %0, %0, %1;" : "+r"(a1) : "r"(b1));
            asm volatile("max.s32 %0, %0, %1;" : "+r"(a2) : "r"(b0));
            asm volatile("max.s32 %0, %0, %1;" : "+r"(a3) : "r"(b1));
            asm volatile("max.s32 %0, %0, %1;" : "+r"(a4) : "r"(b0));
            asm volatile("max.s32 %0, %0, %1;" : "+r"(a5) : "r"(b1));
            asm volatile("max.s32 %0, %0, %1;" : "+r"(a6) : "r"(b0));
            asm volatile("max.s32 %0, %0, %1;" : "+r"(a7) : "r"(b1));
        }
    }
    if ((a0 ^ a1 ^ a2 ^ a3 ^ a4 ^ a5 ^ a6 ^ a7) == 0x7fffffff) out[0] = 1;
}

}  // namespace

int measure_int32_peak(int sm_count, double *tops, cudaStream_t s) {
    int *d = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaError_t e = cudaMalloc(&d, sizeof(int));
    if (e) return (int)e;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int grid = sm_count * 8, block = 256, iters = 4096;
    int32_max_peak_kernel<<<grid, block, 0, s>>>(d, 64, 1);  // warm-up
    cudaEventRecord(e0, s);
    int32_max_peak_kernel<<<grid, block, 0, s>>>(d, iters, 1);
    cudaEventRecord(e1, s);
    e = cudaEventSynchronize(e1);
    float ms = 0;
    if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
    if (!e) *tops = (double)grid * block * iters * 64.0 / (ms * 1e-3) / 1e12;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(d);
    return (int)(e ? e : cudaGetLastError());
}

int launch_sw_forward(const SwArgs &a, int k, const int32_t *tasks, int n_tasks, int *cursor, int grid,
                      cudaStream_t s) {
    if (n_tasks <= 0) return 0;
    switch (k) {
#define GHMM_SW_CASE(KK)                                                                         \
    case KK:                                                                                     \
        if (a.clamp)                                                                             \
            sw_forward_kernel<KK, true><<<grid, 128, 0, s>>>(a, tasks, n_tasks, cursor);         \
        else                                                                                     \
            sw_forward_kernel<KK, false><<<grid, 128, 0, s>>>(a, tasks, n_tasks, cursor);        \
        break;
        GHMM_SW_CASE(1)
        GHMM_SW_CASE(2)
        GHMM_SW_CASE(3)
        GHMM_SW_CASE(4)
        GHMM_SW_CASE(5)
        GHMM_SW_CASE(6)
        GHMM_SW_CASE(7)
        GHMM_SW_CASE(8)
#undef GHMM_SW_CASE
        default: return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}

int sw_forward_occupancy(int k, int *blocks_per_sm) {
    cudaError_t e = cudaErrorInvalidValue;
    switch (k) {
#define GHMM_SW_OCC(KK)                                                                                     \
    case KK: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, sw_forward_kernel<KK, false>, 128, 0); \
        break;
        GHMM_SW_OCC(1)
        GHMM_SW_OCC(2)
        GHMM_SW_OCC(3)
        GHMM_SW_OCC(4)
        GHMM_SW_OCC(5)
        GHMM_SW_OCC(6)
        GHMM_SW_OCC(7)
        GHMM_SW_OCC(8)
#undef GHMM_SW_OCC
        default: break;
    }
    return (int)e;
}

int launch_sw_traceback(const SwArgs &a, int n_pairs, cudaStream_t s) {
    if (n_pairs <= 0) return 0;
    sw_traceback_kernel<<<(n_pairs + 127) / 128, 128, 0, s>>>(a, n_pairs);
    return (int)cudaGetLastError();
}

int launch_sw_compact(const SwArgs &a, int n_pairs, int64_t *starts, int64_t *running, uint32_t *ops, int64_t ops_cap,
                      cudaStream_t s) {
    if (n_pairs <= 0) return 0;
    sw_scan_kernel<<<1, 1024, 0, s>>>(a.n_ops, starts, n_pairs, running);
    sw_gather_kernel<<<(n_pairs + 127) / 128, 128, 0, s>>>(a, starts, ops, ops_cap, n_pairs);
    return (int)cudaGetLastError();
}

int launch_sw_realign_setup(const DevBatch &b, const SwRealignArgs &a, int sm_count, cudaStream_t s) {
    if (a.n_reads <= 0) return 0;
    const int block = 128;
    const int64_t want = (a.n_reads + block - 1) / block;
    const int grid = (int)(want < (int64_t)sm_count * 8 ? want : (int64_t)sm_count * 8);
    sw_realign_setup_kernel<<<grid, block, 0, s>>>(b, a);
    return (int)cudaGetLastError();
}

}  // namespace ghmm
