// sw_host.cpp -- host side of the Smith-Waterman entry points (include/ghmm_sw.h): ghmm_sw_align (the
// SWAlignerNativeBinding.align mirror), ghmm_sw_align_batch and ghmm_batch_realign.
//
// A call flows: validate and marshal (refs deduplicated by address, one pinned plane of refs then alts) -> plan
// chunks so that each chunk's traceback bits fit the traceback buffer (4 bits per cell, 32-bit words per lane and
// step) -> one H2D -> per chunk: the score-recurrence kernels by alt columns per lane (8 .. 1, longest refs first),
// the traceback kernel, the cigar compaction into one device array -> D2H of offsets and counts, then of the ops.
// The realign path takes its sequences and likelihoods from a PairHMM batch already on the device: the host only
// sizes each read's buffers by the longest haplotype of its region, and a setup kernel picks the haplotype.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstdio>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "../../include/ghmm.h"
#include "../../include/ghmm_sw.h"
#include "ghmm_internal.h"
#include "host_util.h"

using namespace ghmm;

namespace ghmm {

struct SwEngine {
    HostBuf<SwPair> h_pairs;
    DevBuf<SwPair> d_pairs;
    HostBuf<int32_t> h_tasks;
    DevBuf<int32_t> d_tasks;
    HostBuf<int2> h_pair_tasks;
    DevBuf<int2> d_pair_tasks;
    HostBuf<uint8_t> h_planes;
    DevBuf<uint8_t> d_planes;
    DevBuf<int32_t> d_res;      // state | offset | n_ops | best, n each
    DevBuf<int64_t> d_starts;
    DevBuf<int64_t> d_block_sums;
    DevBuf<uint32_t> d_ops;
    DevBuf<int64_t> d_counters; // [0] running op total, [1] error flag (as int), then int cursors
    DevBuf<uint32_t> d_tb;
    DevBuf<int> d_edges;
    DevBuf<int2> d_scratch;
    DevBuf<uint32_t> d_slot;
    DevBuf<double> d_prio;
    DevBuf<uint8_t> d_inf;
    HostBuf<int32_t> h_res;
    HostBuf<int64_t> h_starts;
    HostBuf<int64_t> h_counters;
    HostBuf<uint32_t> h_ops;
    std::vector<cudaEvent_t> events;
    ghmm_sw_stats stats{};
    bool allow16 = true;  // pair eligible alignments in the 16-bit kernel
    int64_t tb_budget_words = 0;  // traceback words per chunk; 0: chosen on first use

    cudaEvent_t event(size_t i) {
        while (events.size() <= i) {
            cudaEvent_t e = nullptr;
            cudaEventCreate(&e);
            events.push_back(e);
        }
        return events[i];
    }
    void release() {
        h_pairs.release(); d_pairs.release(); h_tasks.release(); d_tasks.release(); h_planes.release();
        h_pair_tasks.release(); d_pair_tasks.release();
        d_planes.release(); d_res.release(); d_starts.release(); d_ops.release(); d_counters.release();
        d_block_sums.release();
        d_tb.release(); d_edges.release(); d_scratch.release(); d_slot.release(); d_prio.release(); d_inf.release();
        h_res.release(); h_starts.release(); h_counters.release(); h_ops.release();
        for (auto e : events) cudaEventDestroy(e);
        events.clear();
    }
};

void sw_engine_destroy(SwEngine *e) {
    if (!e) return;
    e->release();
    delete e;
}

}  // namespace ghmm

namespace {

#define SW_CUDA(call, what)                                             \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return cuda_error(ctx, e_, what);        \
    } while (0)

int cuda_error(ghmm_ctx *ctx, cudaError_t e, const char *what) {
    return ctx_fail(ctx, e == cudaErrorMemoryAllocation ? GHMM_ERR_NOMEM : GHMM_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(e));
}

constexpr int kCursorsPerChunk = kSwMaxK + 1;

int sw_k(int alt_len) { return alt_len > 32 * kSwMaxK ? kSwMaxK : (alt_len + 31) / 32; }

struct Chunk {
    int64_t p0 = 0, p1 = 0;
    int64_t tb_words = 0, edges = 0, slots = 0, scratch = 0;
    int64_t task_begin[kSwMaxK + 1]{}, task_count[kSwMaxK + 1]{};      // int32 kernel: one alignment per task
    int64_t pair_begin[kSwMaxK + 1]{}, pair_count[kSwMaxK + 1]{};      // 16-bit kernel: two alignments per task
};

// Whether every score of an alignment with a ref of n bases and K alt columns per lane (the lanes' padding columns
// included) stays far inside the 16-bit halves of the paired kernel: scores lie between the best all-diagonal path
// from the matrix edge and max(0, match) per diagonal step (gap penalties only lower a path), gap values between a
// score plus the open penalty and the best score plus it, and the very low initial gap value must still lose to a
// first opening.  Positive gap penalties or large parameters go to the int32 kernel.
bool fits16(const ghmm_sw_params &p, int strategy, int64_t n, int k) {
    const int64_t w = 32 * (int64_t)k;
    const int64_t m = p.match_value, mm = p.mismatch_penalty, o = p.gap_open_penalty, e = p.gap_extend_penalty;
    if (o > 0 || e > 0) return false;
    const int64_t am = std::llabs(m), amm = std::llabs(mm), ao = -o, ae = -e;
    if (am > 2048 || amm > 2048 || ao > 2048 || ae > 2048) return false;
    const int64_t edge_min = (strategy == kSwIndel || strategy == kSwLeadingIndel) ? o + e * (std::max(n, w) - 1) : 0;
    const int64_t diag = std::min(n, w);
    const int64_t hmin = edge_min + std::min<int64_t>({0, m, mm}) * diag;
    const int64_t hmax = std::max<int64_t>(0, m) * diag;
    const int64_t slack = am + amm + ao + ae;
    return hmin - slack >= -28000 && hmax + slack <= 28000;
}

// keys[i]: the alignment's task bucket (kernel * 9 + K) << 21 | ref length, or kNoTask.
constexpr uint32_t kNoTask = 0xffffffffu;

// Buffer sizes of one alignment: traceback words, edge ints, cigar slots, strip scratch rows.
struct SwSizes {
    int64_t words = 0, edges = 0, slots = 0, scratch = 0;
};
inline SwSizes sw_sizes(const SwPair &P, bool runs) {
    SwSizes z;
    z.slots = 2 * (int64_t)P.alt_len + 4;
    if (!runs) return z;
    const int k = sw_k(P.alt_len);
    const int64_t strips = (P.alt_len + 32 * k - 1) / (32 * k);
    z.words = strips * sw_steps4(P.ref_len) * 32;
    z.edges = ((int64_t)P.ref_len + strips * 32) * kSwRowStride(k);  // last-column rows, one bottom row per lane
    z.scratch = strips > 1 ? (int64_t)P.ref_len + 1 : 0;
    return z;
}

struct SwCaps {
    int64_t words, edges, scratch;
};

// The next chunk from alignment i0: buffer offsets (chunk-relative) of every alignment that runs the recurrence
// (state 0, ref_len > 0) and its task key, until one more alignment would pass a buffer's capacity.
Chunk plan_next_chunk(SwPair *pairs, const int32_t *state, int64_t n, int64_t i0, const SwCaps &cap,
                      const ghmm_sw_params &prm, int strategy, bool allow16, std::vector<uint32_t> &keys) {
    Chunk c;
    c.p0 = i0;
    int64_t i = i0;
    for (; i < n; ++i) {
        SwPair &P = pairs[i];
        const bool runs = state[i] == 0 && P.ref_len > 0;
        const SwSizes z = sw_sizes(P, runs);
        if (i > i0 && (c.tb_words + z.words > cap.words || c.edges + z.edges > cap.edges ||
                       c.scratch + z.scratch > cap.scratch))
            break;
        keys[(size_t)i] = kNoTask;
        P.slot_off = c.slots;
        c.slots += z.slots;
        if (!runs) {  // shortcut or nothing to align against: a cigar slot only
            P.k = 1;
            P.tb_off = P.edge_off = 0;
            P.scratch_off = -1;
            continue;
        }
        const int k = sw_k(P.alt_len);
        P.k = k;
        P.tb_off = c.tb_words;
        P.edge_off = c.edges;
        P.scratch_off = z.scratch ? c.scratch : -1;
        c.tb_words += z.words;
        c.edges += z.edges;
        c.scratch += z.scratch;
        const uint32_t kind = allow16 && z.scratch == 0 && fits16(prm, strategy, P.ref_len, k) ? 1u : 0u;
        keys[(size_t)i] = ((kind * (kSwMaxK + 1) + (uint32_t)k) << 21) | (uint32_t)P.ref_len;
    }
    c.p1 = i;
    return c;
}

// One chunk's tasks, at positions p0.. of the task arrays: per K the int32 kernel's alignments (longest ref first)
// and the 16-bit kernel's pairs (neighbours in ref-length order, so the two halves of a warp finish together).  One
// stable counting sort on (kernel, K, descending ref length).  Returns the number of alignments paired.
int64_t plan_tasks(const std::vector<uint32_t> &keys, Chunk &ch, int32_t *tasks, int2 *pair_tasks) {
    constexpr int kBuckets = 2 * (kSwMaxK + 1);
    const uint32_t *kk = keys.data();
    uint32_t lmax = 0;
    for (int64_t i = ch.p0; i < ch.p1; ++i)
        if (kk[i] != kNoTask) lmax = std::max(lmax, kk[i] & 0x1fffffu);
    const int64_t L = (int64_t)lmax + 1;
    std::vector<int32_t> count((size_t)(kBuckets * L + 1), 0);
    auto key = [&](uint32_t x) { return (int64_t)(x >> 21) * L + (int64_t)(lmax - (x & 0x1fffffu)); };
    int64_t runs = 0;
    for (int64_t i = ch.p0; i < ch.p1; ++i)
        if (kk[i] != kNoTask) {
            ++count[(size_t)key(kk[i])];
            ++runs;
        }
    int32_t acc = 0;
    for (auto &c : count) {
        const int32_t x = c;
        c = acc;
        acc += x;
    }
    std::vector<int32_t> bucket_start(kBuckets + 1);
    for (int b = 0; b <= kBuckets; ++b) bucket_start[(size_t)b] = b < kBuckets ? count[(size_t)(b * L)] : (int32_t)runs;
    std::vector<int32_t> order((size_t)std::max<int64_t>(runs, 1));
    for (int64_t i = ch.p0; i < ch.p1; ++i)
        if (kk[i] != kNoTask) order[(size_t)count[(size_t)key(kk[i])]++] = (int32_t)(i - ch.p0);
    int64_t pos = ch.p0, ppos = ch.p0, paired = 0;
    for (int k = kSwMaxK; k >= 1; --k) {  // int32 kernel
        const int32_t b0 = bucket_start[(size_t)k], b1 = bucket_start[(size_t)k + 1];
        ch.task_begin[k] = pos;
        ch.task_count[k] = b1 - b0;
        std::copy(order.begin() + b0, order.begin() + b1, tasks + pos);
        pos += b1 - b0;
    }
    for (int k = kSwMaxK; k >= 1; --k) {  // 16-bit kernel
        const int32_t b0 = bucket_start[(size_t)(kSwMaxK + 1 + k)], b1 = bucket_start[(size_t)(kSwMaxK + 2 + k)];
        ch.pair_begin[k] = ppos;
        ch.pair_count[k] = (b1 - b0 + 1) / 2;
        for (int32_t q = b0; q < b1; q += 2) pair_tasks[ppos++] = make_int2(order[(size_t)q], q + 1 < b1 ? order[(size_t)q + 1] : -1);
        paired += b1 - b0;
    }
    return paired;
}

// Whether any score of these alignments can reach MATRIX_MIN_CUTOFF (or wrap): along the diagonal every score is
// at least the matrix edge it starts from plus min(0, match, mismatch) per cell, and with every quantity far inside
// the int32 range no add wraps.  When that lower bound stays above the cutoff, the clamp never acts.
bool needs_clamp(const ghmm_sw_params &p, int strategy, int64_t max_ref, int64_t max_alt) {
    const int64_t mag = std::llabs((int64_t)p.match_value) + std::llabs((int64_t)p.mismatch_penalty) +
                        std::llabs((int64_t)p.gap_open_penalty) + std::llabs((int64_t)p.gap_extend_penalty);
    const int64_t len = max_ref + max_alt + 2;
    if (mag * len >= (int64_t(1) << 29)) return true;
    int64_t edge_min = 0;
    if (strategy == kSwIndel || strategy == kSwLeadingIndel) {
        const int64_t L = std::max(max_ref, max_alt);
        edge_min = std::min<int64_t>({0, (int64_t)p.gap_open_penalty,
                                      (int64_t)p.gap_open_penalty + (L - 1) * p.gap_extend_penalty});
    }
    const int64_t worst = std::min<int64_t>({0, (int64_t)p.match_value, (int64_t)p.mismatch_penalty});
    return edge_min + worst * std::min(max_ref, max_alt) <= -100000000;
}

struct RunIn {
    const uint8_t *ref_plane, *alt_plane;
    const ghmm_sw_params *params;
    int strategy, shortcut;
    int64_t n;
    int64_t ops_cap;
    // realign: the haplotype of each read is chosen on the device before the chunks are planned
    const BatchInfo *batch = nullptr;
    const double *priority = nullptr;  // host, per batch haplotype
    std::chrono::steady_clock::time_point t0;  // start of the call
};

// Everything after the host pairs hold their sequences: (1) upload, the realign setup and the substring shortcut on
// the device, then the shortcut states (and chosen haplotypes) back to the host; (2) chunk and task planning with
// the exact lengths; (3) per chunk the score kernels, the traceback and the cigar compaction.  On return h_res holds
// state | offset | n_ops | best (n each), h_starts the op starts, h_counters[0] the op total, and h_ops the ops.
int run(ghmm_ctx *ctx, const CtxInfo &ci, SwEngine &E, const RunIn &in, int64_t plane_bytes,
        std::vector<uint8_t> *informative) {
    NvtxRange range("ghmm Smith-Waterman");
    const int64_t n = in.n;
    cudaStream_t s = ci.stream;
    SW_CUDA(E.d_pairs.reserve((size_t)n), "device pairs");
    SW_CUDA(E.d_res.reserve((size_t)n * 4), "device results");
    SW_CUDA(E.d_starts.reserve((size_t)n), "device cigar starts");
    SW_CUDA(E.d_ops.reserve((size_t)std::max<int64_t>(in.ops_cap, 1)), "device cigar ops");
    SW_CUDA(E.h_res.reserve((size_t)n * 4), "pinned results");
    SW_CUDA(E.h_starts.reserve((size_t)n), "pinned starts");
    SW_CUDA(E.h_counters.reserve(2), "pinned counters");
    int32_t *d_state = E.d_res.p, *d_offset = E.d_res.p + n, *d_nops = E.d_res.p + 2 * n, *d_best = E.d_res.p + 3 * n;
    if (plane_bytes > 0)
        SW_CUDA(cudaMemcpyAsync(E.d_planes.p, E.h_planes.p, (size_t)plane_bytes, cudaMemcpyHostToDevice, s),
                "H2D sequences");
    SW_CUDA(cudaMemcpyAsync(E.d_pairs.p, E.h_pairs.p, (size_t)n * sizeof(SwPair), cudaMemcpyHostToDevice, s),
            "H2D pairs");
    E.stats.h2d_bytes = plane_bytes + 2 * n * (int64_t)sizeof(SwPair);
    SwArgs A{};
    A.ref_plane = in.ref_plane;
    A.alt_plane = in.alt_plane;
    A.match = in.params->match_value;
    A.mismatch = in.params->mismatch_penalty;
    A.open = in.params->gap_open_penalty;
    A.extend = in.params->gap_extend_penalty;
    A.strategy = in.strategy;
    A.indel_edges = (in.strategy == kSwIndel || in.strategy == kSwLeadingIndel) ? 1 : 0;
    A.shortcut = in.shortcut && (in.strategy == kSwSoftclip || in.strategy == kSwIgnore) ? 1 : 0;
    A.pairs = E.d_pairs.p;
    A.state = d_state;
    A.offset = d_offset;
    int launches = 0;
    E.stats.ms_host = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - in.t0).count();
    SW_CUDA(cudaEventRecord(E.event(0), s), "event");
    // (1) haplotype choice, substring shortcut
    if (in.batch) {
        SwRealignArgs R{};
        if (in.priority) {
            SW_CUDA(E.d_prio.reserve((size_t)in.batch->n_haps), "device priorities");
            SW_CUDA(cudaMemcpyAsync(E.d_prio.p, in.priority, (size_t)in.batch->n_haps * sizeof(double),
                                    cudaMemcpyHostToDevice, s), "H2D priorities");
            R.priority = E.d_prio.p;
            E.stats.h2d_bytes += in.batch->n_haps * (int64_t)sizeof(double);
        }
        SW_CUDA(E.d_inf.reserve((size_t)n), "device informative flags");
        R.pairs = E.d_pairs.p;
        R.best = d_best;
        R.informative = E.d_inf.p;
        R.first_read = 0;
        R.n_reads = n;
        const int e = launch_sw_realign_setup(*in.batch->dev, R, ci.sm_count, s);
        if (e) return cuda_error(ctx, (cudaError_t)e, "realign setup launch");
        ++launches;
    }
    if (A.shortcut) {
        const int e = launch_sw_prepass(A, (int)n, ci.sm_count, s);
        if (e) return cuda_error(ctx, (cudaError_t)e, "substring shortcut launch");
        ++launches;
    } else {
        SW_CUDA(cudaMemsetAsync(d_state, 0, (size_t)n * sizeof(int32_t), s), "zero states");
    }
    SW_CUDA(cudaEventRecord(E.event(1), s), "event");
    SW_CUDA(cudaMemcpyAsync(E.h_res.p, d_state, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
            "D2H shortcut states");
    if (in.batch)
        SW_CUDA(cudaMemcpyAsync(E.h_res.p + 3 * n, d_best, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
                "D2H chosen haplotypes");
    SW_CUDA(cudaStreamSynchronize(s), "substring shortcut");
    const auto t_plan = std::chrono::steady_clock::now();
    // (2) planning with exact lengths
    if (in.batch) {  // each read's ref is the haplotype chosen on the device
        const int64_t NR = in.batch->n_reads, NH = in.batch->n_haps;
        const int64_t *hap_off = in.batch->h_off + NR + 1, *rro = hap_off + NH + 1, *rho = rro + in.batch->n_regions + 1;
        const int32_t *best = E.h_res.p + 3 * n;
        const int64_t G = in.batch->n_regions;
        parallel_for(G, ci.threads, [&](int64_t g) {
            for (int64_t r = rro[g]; r < rro[g + 1]; ++r) {
                SwPair &P = E.h_pairs.p[r];
                if (best[r] < 0) {
                    P.ref_off = 0;
                    P.ref_len = 0;
                } else {
                    const int64_t h = rho[g] + best[r];
                    P.ref_off = hap_off[h];
                    P.ref_len = (int32_t)(hap_off[h + 1] - hap_off[h]);
                }
            }
        });
    }
    // totals and maxima for the buffers and the clamp decision
    struct Part {
        int64_t words = 0, max_words = 0, max_edges = 0, max_scratch = 0, slots = 0, max_ref = 0, max_alt = 0;
    };
    const int nparts = std::max(1, ci.threads);
    std::vector<Part> parts((size_t)nparts);
    const int64_t per = (n + nparts - 1) / nparts;
    parallel_for(nparts, nparts, [&](int64_t t) {
        Part q;  // (filled locally: neighbouring parts share cache lines)
        for (int64_t i = t * per; i < std::min(n, (t + 1) * per); ++i) {
            const SwPair &P = E.h_pairs.p[i];
            const bool runs = E.h_res.p[i] == 0 && P.ref_len > 0;
            const SwSizes z = sw_sizes(P, runs);
            q.words += z.words;
            q.slots += z.slots;
            q.max_words = std::max(q.max_words, z.words);
            q.max_edges = std::max(q.max_edges, z.edges);
            q.max_scratch = std::max(q.max_scratch, z.scratch);
            if (runs) {
                q.max_ref = std::max<int64_t>(q.max_ref, P.ref_len);
                q.max_alt = std::max<int64_t>(q.max_alt, P.alt_len);
            }
        }
        parts[(size_t)t] = q;
    }, 1);
    Part tot;
    for (auto &q : parts) {
        tot.words += q.words;
        tot.slots += q.slots;
        tot.max_words = std::max(tot.max_words, q.max_words);
        tot.max_edges = std::max(tot.max_edges, q.max_edges);
        tot.max_scratch = std::max(tot.max_scratch, q.max_scratch);
        tot.max_ref = std::max(tot.max_ref, q.max_ref);
        tot.max_alt = std::max(tot.max_alt, q.max_alt);
    }
    A.clamp = needs_clamp(*in.params, in.strategy, tot.max_ref, tot.max_alt) ? 1 : 0;
    // a chunk is bounded by the traceback budget; its edges and scratch by fixed fractions of it (an alignment's
    // edges are at most a quarter of its traceback words and its scratch a 32nd), or by the largest single alignment
    SwCaps cap;
    cap.words = std::max(std::min(E.tb_budget_words, tot.words), tot.max_words);
    cap.edges = std::max(cap.words / 3, tot.max_edges);
    cap.scratch = std::max(cap.words / 16, tot.max_scratch);
    SW_CUDA(E.h_tasks.reserve((size_t)std::max<int64_t>(n, 1)), "pinned tasks");
    SW_CUDA(E.h_pair_tasks.reserve((size_t)std::max<int64_t>(n, 1)), "pinned pair tasks");
    SW_CUDA(E.d_tasks.reserve((size_t)std::max<int64_t>(n, 1)), "device tasks");
    SW_CUDA(E.d_pair_tasks.reserve((size_t)std::max<int64_t>(n, 1)), "device pair tasks");
    SW_CUDA(E.d_counters.reserve((size_t)(2 + kCursorsPerChunk)), "device counters");
    SW_CUDA(E.d_tb.reserve((size_t)std::max<int64_t>(cap.words, 1)), "traceback buffer");
    SW_CUDA(E.d_edges.reserve((size_t)std::max<int64_t>(cap.edges, 4)), "edge scores");
    SW_CUDA(E.d_scratch.reserve((size_t)std::max<int64_t>(cap.scratch, 1)), "strip scratch");
    SW_CUDA(E.d_slot.reserve((size_t)std::max<int64_t>(tot.slots, 1)), "cigar slots");
    SW_CUDA(E.d_block_sums.reserve((size_t)(n / 1024 + 2)), "scan block sums");
    SW_CUDA(cudaMemsetAsync(E.d_counters.p, 0, 2 * sizeof(int64_t), s), "zero counters");
    int *d_err = reinterpret_cast<int *>(E.d_counters.p + 1);
    int *d_cursors = reinterpret_cast<int *>(E.d_counters.p + 2);  // 2 x 9 task cursors, reset per chunk
    A.tb = E.d_tb.p;
    A.edges = E.d_edges.p;
    A.strip_scratch = E.d_scratch.p;
    A.slot = E.d_slot.p;
    A.error = d_err;
    int occ[kSwMaxK + 1]{}, occ16[kSwMaxK + 1]{};
    for (int k = 1; k <= kSwMaxK; ++k) {
        int b = 0, b16 = 0;
        int e = sw_forward_occupancy(k, &b);
        if (!e) e = sw_pair16_occupancy(k, &b16);
        if (e) return cuda_error(ctx, (cudaError_t)e, "occupancy");
        occ[k] = std::max(b, 1);
        occ16[k] = std::max(b16, 1);
    }
    std::vector<uint32_t> keys((size_t)n);
    int64_t n_paired = 0, n_chunks = 0;
    double ms_tasks = 0;
    // the next chunk is planned (offsets and tasks) and uploaded while the previous chunk's kernels run
    auto plan_chunk = [&](int64_t i0, Chunk &ch) -> int {
        const auto t_tasks = std::chrono::steady_clock::now();
        ch = plan_next_chunk(E.h_pairs.p, E.h_res.p, n, i0, cap, *in.params, in.strategy, E.allow16, keys);
        n_paired += plan_tasks(keys, ch, E.h_tasks.p, E.h_pair_tasks.p);
        int64_t nt = 0, np = 0;
        for (int k = 1; k <= kSwMaxK; ++k) {
            nt += ch.task_count[k];
            np += ch.pair_count[k];
        }
        SW_CUDA(cudaMemcpyAsync(E.d_pairs.p + ch.p0, E.h_pairs.p + ch.p0, (size_t)(ch.p1 - ch.p0) * sizeof(SwPair),
                                cudaMemcpyHostToDevice, s), "H2D planned pairs");
        if (nt)
            SW_CUDA(cudaMemcpyAsync(E.d_tasks.p + ch.p0, E.h_tasks.p + ch.p0, (size_t)nt * sizeof(int32_t),
                                    cudaMemcpyHostToDevice, s), "H2D tasks");
        if (np)
            SW_CUDA(cudaMemcpyAsync(E.d_pair_tasks.p + ch.p0, E.h_pair_tasks.p + ch.p0, (size_t)np * sizeof(int2),
                                    cudaMemcpyHostToDevice, s), "H2D pair tasks");
        SW_CUDA(cudaMemsetAsync(d_cursors, 0, 2 * kCursorsPerChunk * sizeof(int), s), "zero task cursors");
        E.stats.h2d_bytes += (ch.p1 - ch.p0) * (int64_t)sizeof(SwPair) + nt * 4 + np * 8;
        ms_tasks += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_tasks).count();
        return GHMM_OK;
    };
    Chunk next;
    if (n > 0) {  // a first chunk of a quarter of the budget starts the GPU sooner; later ones use all of it
        const SwCaps full = cap;
        cap.words = std::max(cap.words / 4, tot.max_words);
        const int rc = plan_chunk(0, next);
        cap = full;
        if (rc) return rc;
    }
    E.stats.ms_host += std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t_plan).count();
    // (3) per chunk
    SW_CUDA(cudaEventRecord(E.event(2), s), "event");
    size_t ev = 3;
    std::vector<std::pair<size_t, size_t>> fwd_events;
    while (n_chunks == 0 || next.p0 < n) {
        const Chunk ch = next;
        ++n_chunks;
        const int64_t cn = ch.p1 - ch.p0;
        SwArgs a = A;
        a.pairs = E.d_pairs.p + ch.p0;
        a.state = d_state + ch.p0;
        a.offset = d_offset + ch.p0;
        a.n_ops = d_nops + ch.p0;
        const size_t e0 = ev++, e1 = ev++;
        SW_CUDA(cudaEventRecord(E.event(e0), s), "event");
        for (int k = kSwMaxK; k >= 1; --k) {
            const int64_t cnt = ch.pair_count[k];
            if (!cnt) continue;
            const int grid = (int)std::min<int64_t>((cnt + 3) / 4, (int64_t)occ16[k] * ci.sm_count);
            const int e = launch_sw_pair16(a, k, E.d_pair_tasks.p + ch.pair_begin[k], (int)cnt,
                                           d_cursors + kCursorsPerChunk + k, grid, s);
            if (e) return cuda_error(ctx, (cudaError_t)e, "Smith-Waterman paired forward launch");
            ++launches;
        }
        for (int k = kSwMaxK; k >= 1; --k) {
            const int64_t cnt = ch.task_count[k];
            if (!cnt) continue;
            const int grid = (int)std::min<int64_t>((cnt + 3) / 4, (int64_t)occ[k] * ci.sm_count);
            const int e = launch_sw_forward(a, k, E.d_tasks.p + ch.task_begin[k], (int)cnt, d_cursors + k, grid, s);
            if (e) return cuda_error(ctx, (cudaError_t)e, "Smith-Waterman forward launch");
            ++launches;
        }
        SW_CUDA(cudaEventRecord(E.event(e1), s), "event");
        fwd_events.emplace_back(e0, e1);
        int e = launch_sw_traceback(a, (int)cn, s);
        if (e) return cuda_error(ctx, (cudaError_t)e, "Smith-Waterman traceback launch");
        e = launch_sw_compact(a, (int)cn, E.d_starts.p + ch.p0, E.d_counters.p, E.d_ops.p, in.ops_cap, E.d_block_sums.p, s);
        if (e) return cuda_error(ctx, (cudaError_t)e, "Smith-Waterman cigar compaction launch");
        launches += 4;
        if (ch.p1 >= n) break;
        const int rc = plan_chunk(ch.p1, next);
        if (rc) return rc;
    }
    const size_t ev_end = ev++;
    SW_CUDA(cudaEventRecord(E.event(ev_end), s), "event");
    SW_CUDA(cudaMemcpyAsync(E.h_res.p + n, d_offset, (size_t)n * 2 * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
            "D2H results");
    SW_CUDA(cudaMemcpyAsync(E.h_starts.p, E.d_starts.p, (size_t)n * sizeof(int64_t), cudaMemcpyDeviceToHost, s),
            "D2H cigar starts");
    SW_CUDA(cudaMemcpyAsync(E.h_counters.p, E.d_counters.p, 2 * sizeof(int64_t), cudaMemcpyDeviceToHost, s),
            "D2H counters");
    if (informative) {
        informative->resize((size_t)n);
        SW_CUDA(cudaMemcpyAsync(informative->data(), E.d_inf.p, (size_t)n, cudaMemcpyDeviceToHost, s),
                "D2H informative flags");
    }
    SW_CUDA(cudaStreamSynchronize(s), "Smith-Waterman kernels");
    E.stats.d2h_bytes = n * (int64_t)(4 * sizeof(int32_t) + sizeof(int64_t)) + 16 + (informative ? n : 0);
    const int err = (int)(E.h_counters.p[1] & 0xffffffff);
    if (err == 2) return ctx_fail(ctx, GHMM_ERR_ARG, "cigar_cap too small for the alignments' cigars");
    if (err) return ctx_fail(ctx, GHMM_ERR_CUDA, "Smith-Waterman traceback overran its buffer");
    const int64_t total = E.h_counters.p[0];
    if (total > in.ops_cap) return ctx_fail(ctx, GHMM_ERR_ARG, "cigar_cap too small for the alignments' cigars");
    SW_CUDA(E.h_ops.reserve((size_t)std::max<int64_t>(total, 1)), "pinned cigar ops");
    if (total > 0) {
        SW_CUDA(cudaMemcpyAsync(E.h_ops.p, E.d_ops.p, (size_t)total * sizeof(uint32_t), cudaMemcpyDeviceToHost, s),
                "D2H cigar ops");
        SW_CUDA(cudaStreamSynchronize(s), "D2H cigar ops");
    }
    E.stats.d2h_bytes += total * (int64_t)sizeof(uint32_t);
    float ms_pre = 0, ms_main = 0;  // device time, without the host planning between the two phases
    cudaEventElapsedTime(&ms_pre, E.event(0), E.event(1));
    cudaEventElapsedTime(&ms_main, E.event(2), E.event(ev_end));
    E.stats.ms_device = ms_pre + ms_main;
    double fwd = 0;
    for (auto &fe : fwd_events) {
        float m = 0;
        cudaEventElapsedTime(&m, E.event(fe.first), E.event(fe.second));
        fwd += m;
    }
    E.stats.ms_forward = fwd;
    E.stats.chunks = (int32_t)n_chunks;
    E.stats.launches = launches;
    E.stats.n_alignments = n;
    E.stats.n_int16 = n_paired;
    E.stats.ms_host += ms_tasks;
    return GHMM_OK;
}

int check_params(ghmm_ctx *ctx, const ghmm_sw_params *params, int32_t strategy) {
    if (!params) return ctx_fail(ctx, GHMM_ERR_ARG, "Smith-Waterman parameters must not be null");
    if (strategy < GHMM_SW_SOFTCLIP || strategy > GHMM_SW_IGNORE)
        return ctx_fail(ctx, GHMM_ERR_ARG, "unknown overhang strategy " + std::to_string(strategy));
    return GHMM_OK;
}

SwEngine *engine(const CtxInfo &ci) {
    if (!*ci.sw) *ci.sw = new SwEngine();
    SwEngine *e = *ci.sw;
    if (e->tb_budget_words == 0) {  // 16 GiB, or a quarter of the free device memory
        size_t free_b = 0, total_b = 0;
        int64_t budget = int64_t(16) << 30;
        if (cudaSetDevice(ci.device) == cudaSuccess && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess)
            budget = std::min<int64_t>(budget, (int64_t)(free_b / 4));
        e->tb_budget_words = std::max<int64_t>(budget, int64_t(1) << 20) / 4;
    }
    return e;
}

// results of pairs [0, n) from the engine's host buffers into the caller's arrays
int deliver(ghmm_ctx *ctx, const CtxInfo &ci, SwEngine &E, int64_t n, const int32_t *ref_len_of,
            ghmm_sw_result *res) {
    const int32_t *state = E.h_res.p, *offset = E.h_res.p + n, *nops = E.h_res.p + 2 * n;
    const int64_t total = E.h_counters.p[0];
    const int parts = std::max(1, ci.threads);
    std::vector<int64_t> n_short((size_t)parts, 0), cells((size_t)parts, 0);
    const int64_t per = (n + parts - 1) / parts;
    parallel_for(parts, parts, [&](int64_t t) {
        int64_t my_short = 0, my_cells = 0;  // (counted locally: neighbouring parts' totals share a cache line)
        for (int64_t i = t * per; i < std::min(n, (t + 1) * per); ++i) {
            res->alignment_offset[i] = offset[i];
            res->cigar_start[i] = E.h_starts.p[i];
            res->cigar_len[i] = nops[i];
            if (ref_len_of && ref_len_of[i] <= 0) continue;  // not aligned
            if (state[i] == 1)
                ++my_short;
            else if (ref_len_of)
                my_cells += (int64_t)ref_len_of[i] * E.h_pairs.p[i].alt_len;
        }
        n_short[(size_t)t] = my_short;
        cells[(size_t)t] = my_cells;
        // this part's share of the cigar ops
        const int64_t o0 = total * t / parts, o1 = total * (t + 1) / parts;
        if (o1 > o0) std::memcpy(res->cigar_ops + o0, E.h_ops.p + o0, (size_t)(o1 - o0) * sizeof(uint32_t));
    }, 1);
    res->cigar_total = total;
    E.stats.n_shortcut = std::accumulate(n_short.begin(), n_short.end(), int64_t(0));
    E.stats.cells = std::accumulate(cells.begin(), cells.end(), int64_t(0));
    (void)ctx;
    return GHMM_OK;
}

// Distinct (address, length) refs of one block of pairs: an open-addressing table that doubles at half load, holding
// each ref's offset in the block's ref bytes.
struct RefSet {
    struct Slot {
        const uint8_t *ref;
        int32_t len;
        int64_t off;  // < 0: empty
    };
    std::vector<Slot> t = std::vector<Slot>(1024, Slot{nullptr, 0, -1});
    size_t used = 0;
    static size_t hash(const uint8_t *r) { return (size_t)(((uint64_t)(uintptr_t)r * 0x9E3779B97F4A7C15ull) >> 17); }
    // the offset of (r, len); absent, it is added at offset `next` and *added is set
    int64_t find_or_add(const uint8_t *r, int32_t len, int64_t next, bool *added) {
        const size_t mask = t.size() - 1;
        size_t h = hash(r) & mask;
        while (t[h].off >= 0) {
            if (t[h].ref == r && t[h].len == len) return t[h].off;
            h = (h + 1) & mask;
        }
        t[h] = Slot{r, len, next};
        *added = true;
        if (2 * ++used > t.size()) grow();
        return next;
    }
    void grow() {
        std::vector<Slot> old(t.size() * 2, Slot{nullptr, 0, -1});
        old.swap(t);
        const size_t mask = t.size() - 1;
        for (const Slot &e : old) {
            if (e.off < 0) continue;
            size_t h = hash(e.ref) & mask;
            while (t[h].off >= 0) h = (h + 1) & mask;
            t[h] = e;
        }
    }
};

int sw_batch(ghmm_ctx *ctx, const CtxInfo &ci, const ghmm_sw_pair *pairs, int64_t n, const ghmm_sw_params *params,
             int32_t strategy, int32_t flags, ghmm_sw_result *res) {
    const auto t0 = std::chrono::steady_clock::now();
    SwEngine &E = *engine(ci);
    E.stats = ghmm_sw_stats{};
    // (1) per block of consecutive pairs, in parallel: the checks, the refs deduplicated by (address, length) (a
    // haplotype shared by many reads is copied once per block), the block's ref and alt bytes
    const int parts = (int)std::max<int64_t>(1, std::min<int64_t>(ci.threads, n / 4096 + 1));
    std::vector<int64_t> ref_off((size_t)n);  // block-relative until (2)
    std::vector<std::vector<int64_t>> uniq((size_t)parts);  // pair index of each distinct ref of a block, in order
    std::vector<int64_t> bad((size_t)parts, -1), ref_bytes_of((size_t)parts, 0), alt_bytes_of((size_t)parts, 0);
    parallel_for(parts, parts, [&](int64_t t) {
        RefSet set;
        int64_t rb = 0, ab = 0;
        for (int64_t i = n * t / parts; i < n * (t + 1) / parts; ++i) {
            const ghmm_sw_pair &p = pairs[i];
            if (!p.ref || !p.alt || p.ref_len <= 0 || p.alt_len <= 0 || p.ref_len > GHMM_SW_MAX_LEN ||
                p.alt_len > GHMM_SW_MAX_LEN) {
                bad[(size_t)t] = i;
                return;
            }
            bool added = false;
            ref_off[(size_t)i] = set.find_or_add(p.ref, p.ref_len, rb, &added);
            if (added) {
                uniq[(size_t)t].push_back(i);
                rb += p.ref_len;
            }
            ab += p.alt_len;
        }
        ref_bytes_of[(size_t)t] = rb;
        alt_bytes_of[(size_t)t] = ab;
    }, 1);
    for (int t = 0; t < parts; ++t) {
        if (bad[(size_t)t] < 0) continue;
        const ghmm_sw_pair &p = pairs[bad[(size_t)t]];
        if (!p.ref || !p.alt || p.ref_len <= 0 || p.alt_len <= 0)
            return ctx_fail(ctx, GHMM_ERR_ARG,
                            "Non-null, non-empty sequences are required for the Smith-Waterman calculation");
        return ctx_fail(ctx, GHMM_ERR_ARG, "sequence longer than GHMM_SW_MAX_LEN");
    }
    std::vector<int64_t> ref_base((size_t)parts + 1, 0), alt_base((size_t)parts + 1, 0);
    for (int t = 0; t < parts; ++t) {
        ref_base[(size_t)t + 1] = ref_base[(size_t)t] + ref_bytes_of[(size_t)t];
        alt_base[(size_t)t + 1] = alt_base[(size_t)t] + alt_bytes_of[(size_t)t];
    }
    const int64_t ref_bytes = ref_base[(size_t)parts];
    const int64_t plane_bytes = ref_bytes + alt_base[(size_t)parts];
    SW_CUDA(cudaSetDevice(ci.device), "cudaSetDevice");
    SW_CUDA(E.h_planes.reserve((size_t)plane_bytes), "pinned sequences");
    SW_CUDA(E.d_planes.reserve((size_t)plane_bytes), "device sequences");
    SW_CUDA(E.h_pairs.reserve((size_t)n), "pinned pairs");
    // (2) per block: its distinct refs and its alts into the pinned planes (refs first, then alts, blocks in order),
    // and the pairs with their offsets
    uint8_t *hp = E.h_planes.p;
    std::vector<int32_t> ref_len((size_t)n);
    parallel_for(parts, parts, [&](int64_t t) {
        const int64_t rb = ref_base[(size_t)t];
        for (const int64_t i : uniq[(size_t)t])
            std::memcpy(hp + rb + ref_off[(size_t)i], pairs[i].ref, (size_t)pairs[i].ref_len);
        int64_t ao = alt_base[(size_t)t];
        for (int64_t i = n * t / parts; i < n * (t + 1) / parts; ++i) {
            const ghmm_sw_pair &p = pairs[i];
            std::memcpy(hp + ref_bytes + ao, p.alt, (size_t)p.alt_len);
            SwPair &P = E.h_pairs.p[i];
            P = SwPair{};
            P.ref_off = rb + ref_off[(size_t)i];
            P.alt_off = ao;
            P.ref_len = p.ref_len;
            P.alt_len = p.alt_len;
            ref_len[(size_t)i] = p.ref_len;
            ao += p.alt_len;
        }
    }, 1);
    RunIn in{};
    in.ref_plane = E.d_planes.p;
    in.alt_plane = E.d_planes.p + ref_bytes;
    in.params = params;
    in.strategy = strategy;
    in.shortcut = (flags & GHMM_SW_SUBSTRING_SHORTCUT) ? 1 : 0;
    in.n = n;
    in.ops_cap = res->cigar_cap;
    in.t0 = t0;
    int rc = run(ctx, ci, E, in, plane_bytes, nullptr);
    if (rc) return rc;
    rc = deliver(ctx, ci, E, n, ref_len.data(), res);
    E.stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

bool valid_result(const ghmm_sw_result *r) {
    return r && r->alignment_offset && r->cigar_start && r->cigar_len && (r->cigar_ops || r->cigar_cap == 0) &&
           r->cigar_cap >= 0;
}

}  // namespace

extern "C" {

int64_t ghmm_sw_cigar_bound(const ghmm_sw_pair *pairs, int32_t n_pairs) {
    if (!pairs || n_pairs <= 0) return 0;
    int64_t b = 0;
    for (int32_t i = 0; i < n_pairs; ++i) b += 2 * (int64_t)std::max(pairs[i].alt_len, 0) + 4;
    return b;
}

int ghmm_sw_align_batch(ghmm_ctx *ctx, const ghmm_sw_pair *pairs, int32_t n_pairs, const ghmm_sw_params *params,
                        int32_t strategy, int32_t flags, ghmm_sw_result *result) {
    CtxInfo ci;
    if (ctx_info(ctx, &ci)) return GHMM_ERR_STATE;
    if (n_pairs < 0 || (n_pairs > 0 && (!pairs || !valid_result(result))))
        return ctx_fail(ctx, GHMM_ERR_ARG, "NULL argument");
    int rc = check_params(ctx, params, strategy);
    if (rc) return rc;
    if (n_pairs == 0) {
        if (result) result->cigar_total = 0;
        return GHMM_OK;
    }
    return sw_batch(ctx, ci, pairs, n_pairs, params, strategy, flags, result);
}

int ghmm_sw_align(ghmm_ctx *ctx, const uint8_t *ref, int32_t ref_len, const uint8_t *alt, int32_t alt_len,
                  const ghmm_sw_params *params, int32_t strategy, char *cigar, int32_t cigar_cap,
                  int32_t *alignment_offset) {
    CtxInfo ci;
    if (ctx_info(ctx, &ci)) return GHMM_ERR_STATE;
    if (!cigar || cigar_cap <= 0 || !alignment_offset) return ctx_fail(ctx, GHMM_ERR_ARG, "NULL argument");
    int rc = check_params(ctx, params, strategy);
    if (rc) return rc;
    if (!ref || !alt || ref_len <= 0 || alt_len <= 0)
        return ctx_fail(ctx, GHMM_ERR_ARG, "Non-null, non-empty sequences are required for the Smith-Waterman calculation");
    ghmm_sw_pair p{ref, alt, ref_len, alt_len};
    std::vector<uint32_t> ops((size_t)2 * alt_len + 4);
    int32_t off = 0, len = 0;
    int64_t start = 0;
    ghmm_sw_result r{&off, &start, &len, ops.data(), (int64_t)ops.size(), 0};
    rc = sw_batch(ctx, ci, &p, 1, params, strategy, 0, &r);
    if (rc) return rc;
    // TextCigarCodec.encode: length then operator per element, "*" for none
    static const char kOps[] = "MIDNSHP=X";
    std::string text;
    for (int32_t q = 0; q < len; ++q) {
        const uint32_t o = ops[(size_t)(start + q)];
        text += std::to_string(o >> 4);
        text += kOps[o & 15u];
    }
    if (text.empty()) text = "*";
    if ((int64_t)text.size() + 1 > cigar_cap) return ctx_fail(ctx, GHMM_ERR_ARG, "cigar buffer too small");
    std::memcpy(cigar, text.c_str(), text.size() + 1);
    *alignment_offset = off;
    return GHMM_OK;
}

int ghmm_batch_realign(ghmm_ctx *ctx, ghmm_batch *batch, const double *hap_priority, const ghmm_sw_params *params,
                       int32_t *best_hap, uint8_t *informative, ghmm_sw_result *result) {
    CtxInfo ci;
    if (ctx_info(ctx, &ci)) return GHMM_ERR_STATE;
    if (!batch || !params) return ctx_fail(ctx, GHMM_ERR_ARG, "NULL argument");
    BatchInfo bi;
    batch_info(batch, &bi);
    if (!bi.has_results) return ctx_fail(ctx, GHMM_ERR_STATE, "run a forward on the batch first");
    const int64_t n = bi.n_reads;
    if (n > 0 && (!best_hap || !informative || !valid_result(result)))
        return ctx_fail(ctx, GHMM_ERR_ARG, "NULL argument");
    if (n == 0) {
        if (result) result->cigar_total = 0;
        return GHMM_OK;
    }
    const auto t0 = std::chrono::steady_clock::now();
    SwEngine &E = *engine(ci);
    E.stats = ghmm_sw_stats{};
    SW_CUDA(cudaSetDevice(ci.device), "cudaSetDevice");
    const int64_t *read_off = bi.h_off;
    SW_CUDA(E.h_pairs.reserve((size_t)n), "pinned pairs");
    // the reads; their haplotypes are chosen on the device (reads of a region without haplotypes are not aligned)
    std::atomic<bool> empty_read{false};
    parallel_for(n, ci.threads, [&](int64_t r) {
        SwPair &P = E.h_pairs.p[r];
        P = SwPair{};
        P.alt_off = read_off[r];
        P.alt_len = (int32_t)(read_off[r + 1] - read_off[r]);
        if (P.alt_len <= 0) empty_read.store(true, std::memory_order_relaxed);
    }, 4096);
    if (empty_read.load())
        return ctx_fail(ctx, GHMM_ERR_ARG, "Non-null, non-empty sequences are required for the Smith-Waterman calculation");
    RunIn in{};
    in.ref_plane = bi.dev->hap_bases;
    in.alt_plane = bi.dev->bases;
    in.params = params;
    in.strategy = kSwSoftclip;
    in.shortcut = 1;
    in.n = n;
    in.ops_cap = result->cigar_cap;
    in.batch = &bi;
    in.priority = hap_priority;
    in.t0 = t0;
    std::vector<uint8_t> inf;
    int rc = run(ctx, ci, E, in, 0, &inf);
    if (rc) return rc;
    const int32_t *best = E.h_res.p + 3 * n;
    std::vector<int32_t> ref_len((size_t)n);
    parallel_for(n, ci.threads, [&](int64_t r) {
        best_hap[r] = best[r];
        informative[r] = inf[(size_t)r];
        ref_len[(size_t)r] = E.h_pairs.p[r].ref_len;  // the chosen haplotype's length (0: not aligned)
    }, 4096);
    rc = deliver(ctx, ci, E, n, ref_len.data(), result);
    E.stats.d2h_bytes += n * (int64_t)sizeof(int32_t);
    E.stats.ms_total = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    return rc;
}

int ghmm_sw_set_options(ghmm_ctx *ctx, int32_t flags) {
    CtxInfo ci;
    if (ctx_info(ctx, &ci)) return GHMM_ERR_STATE;
    engine(ci)->allow16 = !(flags & GHMM_SW_OPT_INT32_ONLY);
    return GHMM_OK;
}

int ghmm_sw_set_traceback_budget(ghmm_ctx *ctx, int64_t bytes) {
    CtxInfo ci;
    if (ctx_info(ctx, &ci)) return GHMM_ERR_STATE;
    engine(ci)->tb_budget_words = std::max<int64_t>(bytes, int64_t(1) << 20) / 4;
    return GHMM_OK;
}

int ghmm_sw_measure_peak(ghmm_ctx *ctx, double *int32_tops) {
    CtxInfo ci;
    if (ctx_info(ctx, &ci)) return GHMM_ERR_STATE;
    if (!int32_tops) return ctx_fail(ctx, GHMM_ERR_ARG, "NULL argument");
    SW_CUDA(cudaSetDevice(ci.device), "cudaSetDevice");
    const int e = measure_int32_peak(ci.sm_count, int32_tops, ci.stream);
    if (e) return cuda_error(ctx, (cudaError_t)e, "int32 peak loop");
    return GHMM_OK;
}

int ghmm_sw_last_stats(ghmm_ctx *ctx, ghmm_sw_stats *stats) {
    CtxInfo ci;
    if (ctx_info(ctx, &ci)) return GHMM_ERR_STATE;
    if (!stats) return ctx_fail(ctx, GHMM_ERR_ARG, "NULL argument");
    *stats = *ci.sw ? (*ci.sw)->stats : ghmm_sw_stats{};
    return GHMM_OK;
}

}  // extern "C"
