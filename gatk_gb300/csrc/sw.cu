// sw.cu -- Smith-Waterman alignment on the device: what GATK's SmithWatermanJavaAligner computes
// (src/main/java/org/broadinstitute/hellbender/utils/smithwaterman/SmithWatermanJavaAligner.java:59-379) and what the
// native SWAlignerNativeBinding.align returns (SWNativeAlignerWrapper.java:31-59): a cigar and an alignment offset
// of `alt` against `ref`, for the four overhang strategies, bit-identical to the Java code.
//
// Pipeline of one batch (all on one stream):
//   sw_prepass_kernel     the exact-substring shortcut (Utils.lastIndexOf, Utils.java:1124-1138), one warp per
//                         alignment, when enabled; the host then plans chunks and tasks with the exact lengths.
//   sw_pair16_kernel<K>   two alignments per warp in the 16-bit halves of each register, for alignments whose scores
//                         provably fit; sw_forward_kernel<K, CLAMP> one alignment per warp in int32 for the rest.
//                         Both run calculateMatrix's recurrence (:109-228) as an anti-diagonal wavefront: lane l owns
//                         K consecutive alt columns, the warp streams over the ref rows, each lane passing its last
//                         column's score and the row's best horizontal gap to the next lane every step.  Alts longer
//                         than 32*K run in strips of 32*K columns (int32 kernel) whose boundary column goes through a
//                         per-pair scratch.  Per cell 4 traceback bits (not diagonal; horizontal >= vertical;
//                         vertical gap opened here; horizontal gap opened here), from which the traceback rebuilds
//                         the backtrack entry 0 / -ki / +kd exactly: a gap's length is the distance to the cell that
//                         opened it.  The last column's and the bottom row's scores go to an edge array.
//   sw_traceback_kernel   one thread per alignment: end cell per strategy, traceback, cigar elements in reverse
//                         into a per-pair slot (calculateCigar, :261-379).
//   sw_scan_*_kernel      exclusive prefix sums of per-pair element counts and the copy into one compact array of
//                         forward-ordered BAM-encoded cigar ops.
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

// K words to a 16-byte-aligned row (K rounded up to whole int4s)
template <int K, typename T>
__device__ __forceinline__ void store_row(int *dst, const T (&w)[K]) {
#pragma unroll
    for (int q = 0; q < K; q += 4)
        reinterpret_cast<int4 *>(dst)[q / 4] =
            make_int4((int)w[q], q + 1 < K ? (int)w[q + 1 < K ? q + 1 : 0] : 0, q + 2 < K ? (int)w[q + 2 < K ? q + 2 : 0] : 0,
                      q + 3 < K ? (int)w[q + 3 < K ? q + 3 : 0] : 0);
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
__device__ __forceinline__ uint32_t sw_step(const StripCtx &C, LaneState<K> &L, int t, int lane) {
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
    if (!active) return 0;
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
    if (C.owns_last) store_row<K>(C.lastrow + (int64_t)(i - 1) * kSwRowStride(K), L.hup);
    if (C.strip_out && lane == 31) C.strip_out[i] = make_int2(hl, bh);
    L.send_h = hl;
    L.send_b = bh;
    L.hdiag = h_left;
    return bits;
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
    C.tb = A.tb + P.tb_off + (int64_t)s * sw_steps4(n) * 32 + lane * 4;
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
    // traceback words: groups of 4 steps per lane, 16 contiguous bytes (steps t and t - 1 of a lane share a sector)
    int t = 0;
    for (; t < 32; ++t) C.tb[(int64_t)(t >> 2) * 128 + (t & 3)] = sw_step<K, CLAMP, true>(C, L, t, lane);
    for (; t + 3 < n; t += 4) {  // every lane inside the matrix
        const uint32_t w0 = sw_step<K, CLAMP, false>(C, L, t, lane);
        const uint32_t w1 = sw_step<K, CLAMP, false>(C, L, t + 1, lane);
        const uint32_t w2 = sw_step<K, CLAMP, false>(C, L, t + 2, lane);
        const uint32_t w3 = sw_step<K, CLAMP, false>(C, L, t + 3, lane);
        *reinterpret_cast<uint4 *>(C.tb + (int64_t)(t >> 2) * 128) = make_uint4(w0, w1, w2, w3);
    }
    for (; t < n + 31; ++t) C.tb[(int64_t)(t >> 2) * 128 + (t & 3)] = sw_step<K, CLAMP, true>(C, L, t, lane);
    // the lanes finish on row n: their scores (+ open) are the bottom row, one row of kSwRowStride(K) per lane
    store_row<K>(A.edges + P.edge_off + ((int64_t)n + s * 32 + lane) * kSwRowStride(K), L.hup);
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
        const SwPair P = A.pairs[tasks[task]];
        const int nstrips = (P.alt_len + 32 * K - 1) / (32 * K);
        for (int s = 0; s < nstrips; ++s) sw_strip<K, CLAMP>(A, P, s, nstrips);
    }
}

// ---- two alignments per lane, in the 16-bit halves of 32-bit registers ----
// Every score is kept as x + 32768 in its half (so unsigned 16-bit maxima order them as signed values), and with
// every half inside [0, 65535] a plain 32-bit add of c * 0x10001 adds c to both halves without a carry or a borrow
// crossing between them.  The host sends a pair here only when a bound on every score of both alignments keeps the
// halves inside that range; the values are then exactly the int32 ones.
constexpr int kSw16Low = -28672;  // the very low initial gap value (Java: Integer.MIN_VALUE / 2) as a 16-bit score

__device__ __forceinline__ uint32_t vmax2(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("max.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
__device__ __forceinline__ uint32_t vmin2(uint32_t a, uint32_t b) {
    uint32_t d;
    asm("min.u16x2 %0, %1, %2;" : "=r"(d) : "r"(a), "r"(b));
    return d;
}
__device__ __forceinline__ uint32_t both16(int x) { return (uint32_t)(x + 32768) * 0x10001u; }
__device__ __forceinline__ uint32_t addc16(int c) { return (uint32_t)c * 0x10001u; }
__device__ __forceinline__ int lo16(uint32_t w) { return (int)(w & 0xffffu) - 32768; }
__device__ __forceinline__ int hi16(uint32_t w) { return (int)(w >> 16) - 32768; }

struct Pair16Ctx {
    const uint8_t *ref_a, *ref_b;
    uint32_t *tb_a, *tb_b;     // this lane's traceback word of step 0 in each alignment's own layout
    int *last_a, *last_b;      // rows of the lane holding each alignment's last column (the lane's raw words)
    int *bottom_a, *bottom_b;  // each alignment's bottom row, this lane's raw words
    int n_a, n_b, n, m_a, m_b, jbase;
    uint32_t ext2, open2, mo2, inject_const;
    int dm, open, ext;
    bool has_b, owns_a, owns_b, indel_edges;
};

template <int K>
struct Lane16 {
    uint32_t b[K];    // alt bases of alignment A (low half) and B (high half)
    uint32_t hup[K];  // H[i-1][j] + open before a step, H[i][j] + open after it
    uint32_t bv[K];
    uint32_t hdiag, send_h, send_b, a_next;
};

template <int K, bool CHECK>
__device__ __forceinline__ uint2 pair16_step(const Pair16Ctx &C, Lane16<K> &L, int t, int lane) {
    const int i = t - lane + 1;
    const bool active = !CHECK || (i >= 1 && i <= C.n);
    const uint32_t a2 = L.a_next;
    L.a_next = (uint32_t)C.ref_a[min(max(i, 0), C.n_a - 1)] | ((uint32_t)C.ref_b[min(max(i, 0), C.n_b - 1)] << 16);
    uint32_t h_left = __shfl_up_sync(0xffffffffu, L.send_h, 1);
    uint32_t bh = __shfl_up_sync(0xffffffffu, L.send_b, 1);
    if (lane == 0) {
        h_left = C.indel_edges && i > 0 ? both16(C.open + (i - 1) * C.ext + C.open) : C.inject_const;
        bh = both16(kSw16Low);
    }
    if (!active) return make_uint2(0, 0);
    uint32_t bits0 = 0, bits1 = 0;
    uint32_t hd = L.hdiag, hl = h_left;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const uint32_t ne = vmin2(a2 ^ L.b[k], 0x00010001u);       // 1 in a half whose bases differ
        const uint32_t diag = ne * (uint32_t)C.dm + hd + C.mo2;      // + match (or mismatch) - open, per half
        const uint32_t bvk = L.bv[k] + C.ext2, pv = L.hup[k];
        const uint32_t v = vmax2(bvk, pv);
        const uint32_t bhk = bh + C.ext2, ph = hl;
        const uint32_t h = vmax2(bhk, ph);
        const uint32_t g = vmax2(h, v);
        const uint32_t hn = vmax2(diag, g);
        // flags as 0/1 per half (each difference is >= 0 in both halves), placed at bit 4(k%4)+f of each half
        const uint32_t f0 = vmin2(hn - diag, 0x00010001u);  // not diagonal
        const uint32_t f1 = vmin2(g - h, 0x00010001u);      // right < down (flipped below)
        const uint32_t f2 = vmin2(v - bvk, 0x00010001u);    // vertical gap opened here
        const uint32_t f3 = vmin2(h - bhk, 0x00010001u);    // horizontal gap opened here
        uint32_t &w = k < 4 ? bits0 : bits1;
        const int sh = 4 * (k & 3);
        w += f0 << sh;
        w += f1 << (sh + 1);
        w += f2 << (sh + 2);
        w += f3 << (sh + 3);
        const uint32_t hno = hn + C.open2;
        L.bv[k] = v;
        bh = h;
        hd = L.hup[k];
        L.hup[k] = hno;
        hl = hno;
    }
    // each alignment's word in the int32 kernel's layout (bit 1 there: right >= down)
    const uint32_t wa = __byte_perm(bits0, bits1, 0x5410) ^ 0x22222222u;
    const uint32_t wb = __byte_perm(bits0, bits1, 0x7632) ^ 0x22222222u;
    // raw 16-bit pairs; the traceback takes its alignment's half (state 2: low, 3: high)
    if (C.owns_a && i <= C.n_a) store_row<K>(C.last_a + (int64_t)(i - 1) * kSwRowStride(K), L.hup);
    if (C.owns_b && i <= C.n_b) store_row<K>(C.last_b + (int64_t)(i - 1) * kSwRowStride(K), L.hup);
    if (i == C.n_a) store_row<K>(C.bottom_a, L.hup);
    if (C.has_b && i == C.n_b) store_row<K>(C.bottom_b, L.hup);
    L.send_h = hl;
    L.send_b = bh;
    L.hdiag = h_left;
    return make_uint2(wa, wb);
}

// tasks: (alignment A, alignment B or -1) of single-strip alignments with the same K, B's ref no longer than A's
template <int K>
__global__ void __launch_bounds__(128, 6) sw_pair16_kernel(SwArgs A, const int2 *tasks, int n_tasks, int *cursor) {
    const int lane = threadIdx.x & 31;
    for (;;) {
        int task = 0;
        if (lane == 0) task = atomicAdd(cursor, 1);
        task = __shfl_sync(0xffffffffu, task, 0);
        if (task >= n_tasks) break;
        const int2 tk = tasks[task];
        const SwPair PA = A.pairs[tk.x];
        const bool has_b = tk.y >= 0;
        const SwPair PB = has_b ? A.pairs[tk.y] : PA;
        Pair16Ctx C;
        C.ref_a = A.ref_plane + PA.ref_off;
        C.ref_b = A.ref_plane + PB.ref_off;
        C.n_a = PA.ref_len;
        C.n_b = PB.ref_len;
        C.n = max(C.n_a, C.n_b);
        C.m_a = PA.alt_len;
        C.m_b = PB.alt_len;
        C.jbase = lane * K;
        C.has_b = has_b;
        C.open = A.open;
        C.ext = A.extend;
        C.ext2 = addc16(A.extend);
        C.open2 = addc16(A.open);
        C.mo2 = addc16(A.match - A.open);
        C.dm = A.mismatch - A.match;
        C.indel_edges = A.indel_edges != 0;
        C.inject_const = both16(A.open);
        C.tb_a = A.tb + PA.tb_off + lane * 4;
        C.tb_b = A.tb + PB.tb_off + lane * 4;
        const int km_a = (C.m_a - 1) - C.jbase, km_b = (C.m_b - 1) - C.jbase;
        C.owns_a = km_a >= 0 && km_a < K;
        C.owns_b = has_b && km_b >= 0 && km_b < K;
        C.last_a = A.edges + PA.edge_off;
        C.last_b = A.edges + PB.edge_off;
        C.bottom_a = A.edges + PA.edge_off + ((int64_t)C.n_a + lane) * kSwRowStride(K);
        C.bottom_b = A.edges + PB.edge_off + ((int64_t)C.n_b + lane) * kSwRowStride(K);
        if (lane == 0) {
            A.state[tk.x] = 2;
            if (has_b) A.state[tk.y] = 3;
        }
        const uint8_t *alt_a = A.alt_plane + PA.alt_off, *alt_b = A.alt_plane + PB.alt_off;
        Lane16<K> L;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int j = C.jbase + k + 1;
            const uint32_t ba = j <= C.m_a ? alt_a[j - 1] : 0u, bb = j <= C.m_b ? alt_b[j - 1] : 0u;
            L.b[k] = ba | (bb << 16);
            L.hup[k] = both16(edge_init(A, j) + A.open);
            L.bv[k] = both16(kSw16Low);
        }
        L.hdiag = both16(edge_init(A, C.jbase) + A.open);
        L.send_h = 0;
        L.send_b = both16(kSw16Low);
        L.a_next = (uint32_t)C.ref_a[0] | ((uint32_t)C.ref_b[0] << 16);
        if (lane > 0) L.a_next = 0;  // lanes start later; their first base is loaded by their own steps
        // each alignment's words for its own n + 31 steps, in groups of 4 steps per lane
        auto put1 = [&](int t, uint2 w) {
            const int64_t o = (int64_t)(t >> 2) * 128 + (t & 3);
            if (t < C.n_a + 31) C.tb_a[o] = w.x;
            if (C.has_b && t < C.n_b + 31) C.tb_b[o] = w.y;
        };
        int t = 0;
        for (; t < 32; ++t) put1(t, pair16_step<K, true>(C, L, t, lane));
        for (; t + 3 < C.n; t += 4) {  // every lane inside the matrix
            const uint2 w0 = pair16_step<K, false>(C, L, t, lane);
            const uint2 w1 = pair16_step<K, false>(C, L, t + 1, lane);
            const uint2 w2 = pair16_step<K, false>(C, L, t + 2, lane);
            const uint2 w3 = pair16_step<K, false>(C, L, t + 3, lane);
            const int64_t o = (int64_t)(t >> 2) * 128;
            if (t + 3 < C.n_a + 31) {
                *reinterpret_cast<uint4 *>(C.tb_a + o) = make_uint4(w0.x, w1.x, w2.x, w3.x);
            } else {
                put1(t, make_uint2(w0.x, 0));
            }
            if (C.has_b) {
                if (t + 3 < C.n_b + 31) {
                    *reinterpret_cast<uint4 *>(C.tb_b + o) = make_uint4(w0.y, w1.y, w2.y, w3.y);
                } else {
                    if (t < C.n_b + 31) C.tb_b[o] = w0.y;
                    if (t + 1 < C.n_b + 31) C.tb_b[o + 1] = w1.y;
                    if (t + 2 < C.n_b + 31) C.tb_b[o + 2] = w2.y;
                }
            }
        }
        for (; t < C.n + 31; ++t) put1(t, pair16_step<K, true>(C, L, t, lane));
        __syncwarp();
    }
}

// The exact-substring shortcut (Utils.lastIndexOf) of every alignment, one warp each, before the recurrence:
// state 1 and the offset for an alt found in its ref, state 0 otherwise (and for every alignment when off).
__global__ void __launch_bounds__(128) sw_prepass_kernel(SwArgs A, int n_pairs) {
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x / 32);
    for (int p = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); p < n_pairs; p += warps) {
        const SwPair P = A.pairs[p];
        int idx = -1;
        if (A.shortcut && P.ref_len > 0)
            idx = warp_last_index_of(A.ref_plane + P.ref_off, P.ref_len, A.alt_plane + P.alt_off, P.alt_len);
        if (lane == 0) {
            A.state[p] = idx >= 0 ? 1 : 0;
            if (idx >= 0) A.offset[p] = idx;
        }
    }
}

// traceback bits of cell (i, j), 1-based
// Traceback bits of cell (i, j), 1-based.  Keeps the last 16-byte group (4 steps of one lane) it loaded: walks move
// one step back per cell along a lane, so most cells come from the group already held.
struct TbReader {
    const uint32_t *base;  // the alignment's words
    int64_t strip_words;
    int K;
    int64_t held = -1;     // word index of the group held
    uint4 g;
    __device__ __forceinline__ uint32_t code(int i, int j) {
        const int w = 32 * K;
        const int s = (j - 1) / w, within = (j - 1) - s * w;
        const int lane = within / K, k = within - lane * K;
        const int64_t t = (int64_t)(i - 1) + lane;
        const int64_t grp = (int64_t)s * strip_words + ((t >> 2) * 32 + lane) * 4;
        if (grp != held) {
            g = *reinterpret_cast<const uint4 *>(base + grp);
            held = grp;
        }
        const int q = (int)(t & 3);
        const uint32_t word = q == 0 ? g.x : q == 1 ? g.y : q == 2 ? g.z : g.w;
        return (word >> (4 * k)) & 15u;
    }
};

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
    const int st = A.state[p];              // 0: int32 scores; 2 / 3: 16-bit pairs, low / high half
    const int *lastcol = A.edges + P.edge_off + km, *bottom = A.edges + P.edge_off + (int64_t)n * stride;
    // a stored score (H + open, or its biased 16-bit half) back to H
    auto score = [&](int w) -> int {
        if (st == 2) w = lo16((uint32_t)w);
        else if (st == 3) w = hi16((uint32_t)w);
        return wsub(w, A.open);
    };
    int p1 = 0, p2 = 0;
    int maxscore = INT32_MIN;
    int segment = 0;
    if (A.strategy == kSwIndel) {
        p1 = n;
        p2 = m;
    } else {
        p2 = m;
        for (int i = 1; i <= n; ++i) {
            const int sc = score(lastcol[(int64_t)(i - 1) * stride]);
            if (sc >= maxscore) {
                p1 = i;
                maxscore = sc;
            }
        }
        if (A.strategy != kSwLeadingIndel) {
            for (int j = 1; j <= m; ++j) {
                const int sc = score(bottom[(int64_t)((j - 1) / K) * stride + (j - 1) % K]);
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
    TbReader rd;
    rd.base = A.tb + P.tb_off;
    rd.strip_words = sw_steps4(n) * 32;
    rd.K = K;
    int state = kSwOpM;
    int guard = n + m + 2;
    do {
        const uint32_t c = rd.code(p1, p2);
        int ns, step = 1;
        if (!(c & 1u)) {
            ns = kSwOpM;
        } else if (c & 2u) {  // horizontal: the gap's length is the distance back to the cell that opened it
            ns = kSwOpI;
            int q = p2;
            while (q > 1 && !(rd.code(p1, q) & 8u)) --q;
            step = p2 - q + 1;
        } else {              // vertical
            ns = kSwOpD;
            int r = p1;
            while (r > 1 && !(rd.code(r, p2) & 4u)) --r;
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

// Cigar compaction: exclusive prefix sums of the chunk's op counts, starting at *running (which then advances by
// their sum), and the reversed per-pair slots copied out in forward order.  Three kernels: per-block sums of 1024
// counts, one block scanning those sums, and a per-block scan plus the copy.
constexpr int kScanBlock = 1024;

__device__ __forceinline__ int64_t block_exclusive_scan(int64_t v, int64_t *sh, int64_t *total) {
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    int64_t x = v;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
        const int64_t y = __shfl_up_sync(0xffffffffu, x, d);
        if (lane >= d) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int64_t w = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int64_t y = __shfl_up_sync(0xffffffffu, w, d);
            if (lane >= d) w += y;
        }
        sh[lane] = w;
    }
    __syncthreads();
    const int64_t before = (warp > 0 ? sh[warp - 1] : 0) + x - v;
    if (total) *total = sh[(blockDim.x >> 5) - 1];
    return before;
}

__global__ void __launch_bounds__(kScanBlock) sw_scan_partials_kernel(const int32_t *counts, int64_t n,
                                                                      int64_t *block_sums) {
    __shared__ int64_t sh[32];
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    const int64_t v = i < n ? counts[i] : 0;
    int64_t tot = 0;
    block_exclusive_scan(v, sh, &tot);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = tot;
}

// one block: exclusive scan of the block sums in chunks of 1024, offset by *running, which advances
__global__ void __launch_bounds__(kScanBlock) sw_scan_blocks_kernel(int64_t *block_sums, int64_t nb, int64_t *running) {
    __shared__ int64_t sh[32];
    __shared__ int64_t carry;
    if (threadIdx.x == 0) carry = *running;
    __syncthreads();
    for (int64_t b0 = 0; b0 < nb; b0 += kScanBlock) {
        const int64_t b = b0 + threadIdx.x;
        const int64_t v = b < nb ? block_sums[b] : 0;
        int64_t tot = 0;
        const int64_t before = block_exclusive_scan(v, sh, &tot);
        if (b < nb) block_sums[b] = carry + before;
        __syncthreads();
        if (threadIdx.x == 0) carry += tot;
        __syncthreads();
    }
    if (threadIdx.x == 0) *running = carry;
}

__global__ void __launch_bounds__(kScanBlock) sw_scan_gather_kernel(SwArgs A, const int64_t *block_sums,
                                                                    int64_t *starts, uint32_t *ops, int64_t ops_cap,
                                                                    int64_t n) {
    __shared__ int64_t sh[32];
    const int64_t i = (int64_t)blockIdx.x * kScanBlock + threadIdx.x;
    const int c = i < n ? A.n_ops[i] : 0;
    const int64_t st = block_sums[blockIdx.x] + block_exclusive_scan(c, sh, nullptr);
    if (i >= n) return;
    starts[i] = st;
    if (st + c > ops_cap) {
        atomicExch(A.error, 2);
        return;
    }
    const uint32_t *slot = A.slot + A.pairs[i].slot_off;
    uint32_t *o = ops + st;
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

int launch_sw_pair16(const SwArgs &a, int k, const int2 *tasks, int n_tasks, int *cursor, int grid, cudaStream_t s) {
    if (n_tasks <= 0) return 0;
    switch (k) {
#define GHMM_SW16_CASE(KK) \
    case KK: sw_pair16_kernel<KK><<<grid, 128, 0, s>>>(a, tasks, n_tasks, cursor); break;
        GHMM_SW16_CASE(1)
        GHMM_SW16_CASE(2)
        GHMM_SW16_CASE(3)
        GHMM_SW16_CASE(4)
        GHMM_SW16_CASE(5)
        GHMM_SW16_CASE(6)
        GHMM_SW16_CASE(7)
        GHMM_SW16_CASE(8)
#undef GHMM_SW16_CASE
        default: return (int)cudaErrorInvalidValue;
    }
    return (int)cudaGetLastError();
}

int sw_pair16_occupancy(int k, int *blocks_per_sm) {
    cudaError_t e = cudaErrorInvalidValue;
    switch (k) {
#define GHMM_SW16_OCC(KK) \
    case KK: e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, sw_pair16_kernel<KK>, 128, 0); break;
        GHMM_SW16_OCC(1)
        GHMM_SW16_OCC(2)
        GHMM_SW16_OCC(3)
        GHMM_SW16_OCC(4)
        GHMM_SW16_OCC(5)
        GHMM_SW16_OCC(6)
        GHMM_SW16_OCC(7)
        GHMM_SW16_OCC(8)
#undef GHMM_SW16_OCC
        default: break;
    }
    return (int)e;
}

int launch_sw_prepass(const SwArgs &a, int n_pairs, int sm_count, cudaStream_t s) {
    if (n_pairs <= 0) return 0;
    const int64_t want = ((int64_t)n_pairs + 3) / 4;
    const int grid = (int)(want < (int64_t)sm_count * 16 ? want : (int64_t)sm_count * 16);
    sw_prepass_kernel<<<grid, 128, 0, s>>>(a, n_pairs);
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
                      int64_t *block_sums, cudaStream_t s) {
    if (n_pairs <= 0) return 0;
    const int64_t nb = ((int64_t)n_pairs + kScanBlock - 1) / kScanBlock;
    sw_scan_partials_kernel<<<(unsigned)nb, kScanBlock, 0, s>>>(a.n_ops, n_pairs, block_sums);
    sw_scan_blocks_kernel<<<1, kScanBlock, 0, s>>>(block_sums, nb, running);
    sw_scan_gather_kernel<<<(unsigned)nb, kScanBlock, 0, s>>>(a, block_sums, starts, ops, ops_cap, n_pairs);
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
