// runtime.cpp -- host runtime and C-ABI of the GB300 PairHMM (include/ghmm.h).
//
// A call flows: marshal (multi-threaded copy of every read's five byte arrays and every haplotype into
// pinned planes, haplotype column codes, validation) -> build warp tasks (reads paired within a region
// by rows-per-lane bucket, longest first) -> async H2D -> FP32 bucket launches -> FP64 queue launch ->
// D2H -> validation of results (log10 L <= 0, not NaN; PairHMM.java:305-306).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ghmm.h"
#include "ghmm_internal.h"
#include "host_util.h"
#include "tables.h"

using namespace ghmm;

namespace ghmm {
std::atomic<int64_t> g_refuse_allocations{0};
}

namespace {

std::mutex g_init_error_mu;
std::string g_init_error;

constexpr int kBlock = 128;
constexpr int kWarpsPerBlock = kBlock / 32;
// Default of ghmm_tuning.route_fp64_below: the FP32 pass can represent log10 L down to about -64 (the rerun
// threshold); a read expected 36 decades below that goes to FP64 without trying.
constexpr int kRouteFp64Log10 = -100;

uint8_t base_code(uint8_t b) {
    switch (b) {
        case 'A': return 1;
        case 'C': return 2;
        case 'G': return 4;
        case 'T': return 8;
        case 'N': return 15;
        default: return 0;
    }
}

// column-code base index of a haplotype byte (A, C, G, T, N = 0..4; anything else routes to FP64)
uint8_t base_index(uint8_t b) {
    switch (b) {
        case 'A': return 0;
        case 'C': return 1;
        case 'G': return 2;
        case 'T': return 3;
        default: return 4;
    }
}

struct Bucket {
    int key;  // rows-per-lane | 16 if multi-strip
    int begin, count;
    int grid;
};

}  // namespace

struct ghmm_batch {
    // host (pinned) staging
    HostBuf<uint8_t> h_planes;  // 5 planes back to back
    HostBuf<uint8_t> h_hap;     // raw bytes, kCodePad bytes, codes, kCodePad bytes
    HostBuf<int64_t> h_off;     // read_off | hap_off | region_read_off | region_hap_off | out_off
    HostBuf<int32_t> h_read_region;
    HostBuf<float> h_init_f;
    HostBuf<double> h_init_d;
    HostBuf<F32Task> h_tasks;
    HostBuf<PairRef> h_direct;    // FP32 mode: pairs routed to FP64, rescaled tier then exact tier
    HostBuf<PairRef> h_fp64all;   // FP64 mode: every pair, rescaled tier then exact tier
    HostBuf<double> h_out;
    HostBuf<int32_t> h_counters;  // [kNumCounters] counters, then [2 * kNumBucketKeys] bucket info
    HostBuf<int64_t> h_nout;
    // device
    DevBuf<uint8_t> d_planes, d_hap;
    DevBuf<int64_t> d_off;
    DevBuf<int32_t> d_read_region;
    DevBuf<float> d_init_f;
    DevBuf<double> d_init_d;
    DevBuf<F32Task> d_tasks;
    DevBuf<PairRef> d_rerun;
    DevBuf<double> d_out;
    DevBuf<int32_t> d_counters;  // same layout as h_counters
    DevBuf<int64_t> d_nout;
    DevBuf<uint8_t> d_post;  // postprocess: reference haplotype per region, keep flags per read
    HostBuf<int32_t> h_mapq;  // raw-read batches: mapping quality per read
    DevBuf<int32_t> d_mapq;
    HostBuf<double> h_dragstr;  // raw-read batches with the DRAGstr imputation: GOP then GCP table
    DevBuf<double> d_dragstr;
    // PD-HMM batches: PD flags then state codes per haplotype column (pd.cu)
    HostBuf<uint8_t> h_pd;
    DevBuf<uint8_t> d_pd;
    bool has_pd = false;
    PdPlanes pd{};
    DevBuf<float2> d_scratch32;
    DevBuf<double> d_scratch64;
    // sizes
    int64_t n_regions = 0, n_reads = 0, n_haps = 0, read_bytes = 0, hap_bytes = 0, n_out = 0;
    int64_t n_cells = 0;
    int max_read_len = 0, max_hap_len = 0;
    std::vector<int> region_max_read;  // for the plain kernel's shared-memory size
    // tasks
    std::vector<Bucket> buckets;
    int64_t n_tasks = 0, n_direct = 0, n_direct_exact = 0;
    int64_t cells_direct = 0;  // cells of the pairs sent to FP64 directly
    double ms_host_copy = 0, ms_host_tasks = 0;  // host time of the last marshal: copy + checks, task building
    int64_t n_direct_fp64mode = 0, n_fp64mode_exact = 0;
    std::vector<uint8_t> read_exact;  // reads whose pairs go to the exact FP64 tier directly
    int64_t scratch32_cols = 0;
    int fp64_grid = 0;
    // last forward
    int last_mode = -1;
    int last_launches = 0;
    int64_t last_rerun = 0, last_exact = 0;
    double ms_fp32 = 0, ms_fp64 = 0, ms_plain = 0, ms_total = 0;
    int64_t upload_bytes = 0, forward_h2d = 0, forward_d2h = 0, results_d2h = 0;
    bool uploaded = false;
    DevBatch dev{};
    // asynchronous forward: events of the last enqueue, and the captured launch sequence
    cudaEvent_t ev[5]{};
    bool events_ready = false;
    cudaEvent_t ev_prep[2]{};  // around the read preparation kernels of a raw batch's upload
    bool prep_events = false, prep_timed = false;
    int64_t pending_n_pre = 0;
    int pending_mode = -1;
    cudaGraphExec_t graph[2]{};  // captured FP32 phase and FP64 phase
    std::vector<unsigned char> graph_sig;  // DevBatch bytes, mode, bucket keys and grids the graphs were captured for

    void release() {
        for (auto &g : graph) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
        graph_sig.clear();
        if (events_ready)
            for (auto &e : ev) cudaEventDestroy(e);
        events_ready = false;
        if (prep_events)
            for (auto &e : ev_prep) cudaEventDestroy(e);
        prep_events = prep_timed = false;
        h_nout.release();
        d_nout.release();
        h_planes.release(); h_hap.release(); h_off.release(); h_read_region.release(); h_init_f.release();
        h_init_d.release(); h_tasks.release(); h_direct.release(); h_fp64all.release(); h_out.release(); h_counters.release();
        d_planes.release(); d_hap.release(); d_off.release(); d_read_region.release(); d_init_f.release();
        d_init_d.release(); d_tasks.release(); d_rerun.release(); d_out.release(); d_counters.release();
        d_scratch32.release(); d_scratch64.release(); d_post.release(); h_pd.release(); d_pd.release();
        h_mapq.release(); d_mapq.release(); h_dragstr.release(); d_dragstr.release();
        has_pd = false;
    }
};

struct ghmm_ctx {
    int64_t debug_force_rerun = 0;  // test hook: every n-th FP32 output rerun in FP64 (batches uploaded afterwards)
    int device = 0;
    int sm_count = 0;
    int max_threads = 0;
    bool double_precision = false;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev[8]{};
    DevTables tables{};
    void *table_mem = nullptr;
    HostTables *host_tables = nullptr;  // host copy, for routing decisions
    std::string last_error;
    ghmm_batch scratch_batch;  // reused by the one-shot entry points
    ghmm_batch pd_batch;       // reused by the one-shot PD-HMM entry points
    int max_k = kMaxK32, max_k_multi = kMaxK32, chunk_cols = 16384;
    // Reads whose expected log10 prior product (sum over positions of the per-quality expectation below) is under
    // route_fp64_log10 go to the FP64 kernel directly: their FP32 results would fall below the rerun threshold and
    // be recomputed there anyway, so the FP32 pass over them would be wasted.  A wrong guess costs only time.
    int route_fp64_log10 = kRouteFp64Log10;
    double expect_log10_prior[256] = {};  // (1 - e) log10(1 - e) + e log10(e / 3), e = 10^(-q/10)
    // calibration scratch (checkpointed fronts per resident warp), FP64-redo flags, unit weights
    DevBuf<uint8_t> calib_scratch;
    DevBuf<int> calib_flags;
    DevBuf<double> calib_ones;
    ghmm_queue *pipe = nullptr;      // the queue that pipelines large synchronous calls
    std::atomic<int> open_queues{0};  // queues of this context not yet destroyed (including pipe)
    SwEngine *sw = nullptr;          // Smith-Waterman buffers (sw_host.cpp), created on first use
    bool alive = false;
};

namespace {

// A queue's worker thread reports into the queue's own message instead of the context's, which belongs to
// the caller's thread.
thread_local std::string *t_error_sink = nullptr;

int fail(ghmm_ctx *ctx, int code, const std::string &msg) {
    if (t_error_sink)
        *t_error_sink = msg;
    else if (ctx)
        ctx->last_error = msg;
    return code;
}

int cuda_fail(ghmm_ctx *ctx, cudaError_t e, const char *what) {
    std::string m = std::string(what) + ": " + cudaGetErrorString(e);
    return fail(ctx, e == cudaErrorMemoryAllocation ? GHMM_ERR_NOMEM : GHMM_ERR_CUDA, m);
}

#define GHMM_CUDA(call, what)                         \
    do {                                              \
        cudaError_t e__ = (call);                     \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, what); \
    } while (0)

// Input view shared by the region-array and flat entry points.
// Routing of reads whose gap penalties are only known after the device imputation (DRAGstr).  The checks that
// guard against wrong finite results (a continuation penalty of 0, a matchToMatch probability of about 0) are
// decided for the whole batch from every value the imputation tables can produce.  The growth checks only save
// work: a pair whose rescaled FP32 or FP64 state overflows sums to a non-finite value and moves on to the next tier.
struct RouteBound {
    uint8_t force = 0;  // flags every read gets (bit0 FP64, bit2 exact FP64 tier)
};

struct Source {
    // either regions (per-read pointers) ...
    const ghmm_region *regions = nullptr;
    int64_t n_regions = 0;
    // ... or flat planes
    const ghmm_flat *flat = nullptr;
    const RouteBound *bound = nullptr;  // set when the device rewrites the gap penalties after the upload
};

// Sizes + offsets (pass 1).  Returns error code.
int plan_sizes(ghmm_ctx *ctx, const Source &src, ghmm_batch &b, std::vector<int64_t> &read_off,
               std::vector<int64_t> &hap_off, std::vector<int64_t> &rro, std::vector<int64_t> &rho,
               std::vector<int64_t> &oo) {
    const int64_t G = src.n_regions;
    rro.assign((size_t)G + 1, 0);
    rho.assign((size_t)G + 1, 0);
    oo.assign((size_t)G + 1, 0);
    if (src.flat) {
        const ghmm_flat *f = src.flat;
        for (int64_t g = 0; g <= G; g++) {
            rro[(size_t)g] = f->region_read_off[g] - f->region_read_off[0];
            rho[(size_t)g] = f->region_hap_off[g] - f->region_hap_off[0];
        }
        const int64_t nr = rro[(size_t)G], nh = rho[(size_t)G];
        read_off.resize((size_t)nr + 1);
        hap_off.resize((size_t)nh + 1);
        const int64_t r0 = f->region_read_off[0], h0 = f->region_hap_off[0];
        for (int64_t r = 0; r <= nr; r++) read_off[(size_t)r] = f->read_off[r0 + r] - f->read_off[r0];
        for (int64_t h = 0; h <= nh; h++) hap_off[(size_t)h] = f->hap_off[h0 + h] - f->hap_off[h0];
    } else {
        int64_t nr = 0, nh = 0;
        for (int64_t g = 0; g < G; g++) {
            const ghmm_region &rg = src.regions[g];
            if (rg.n_reads < 0 || rg.n_haps < 0) return fail(ctx, GHMM_ERR_ARG, "negative read or haplotype count");
            if ((rg.n_reads > 0 && !rg.reads) || (rg.n_haps > 0 && !rg.haps))
                return fail(ctx, GHMM_ERR_ARG, "NULL read or haplotype array");
            nr += rg.n_reads;
            nh += rg.n_haps;
            rro[(size_t)g + 1] = nr;
            rho[(size_t)g + 1] = nh;
        }
        read_off.resize((size_t)nr + 1);
        hap_off.resize((size_t)nh + 1);
        read_off[0] = 0;
        hap_off[0] = 0;
        int64_t ri = 0, hi = 0;
        for (int64_t g = 0; g < G; g++) {
            const ghmm_region &rg = src.regions[g];
            for (int32_t r = 0; r < rg.n_reads; r++, ri++) {
                const ghmm_read &rd = rg.reads[r];
                if (rd.length < 0 || rd.length > kMaxReadLen) return fail(ctx, GHMM_ERR_ARG, "read length out of range");
                if (rd.length > 0 && (!rd.bases || !rd.quals || !rd.ins_gop || !rd.del_gop || !rd.gcp))
                    return fail(ctx, GHMM_ERR_ARG, "NULL read array");
                read_off[(size_t)ri + 1] = read_off[(size_t)ri] + rd.length;
            }
            for (int32_t h = 0; h < rg.n_haps; h++, hi++) {
                const ghmm_hap &hp = rg.haps[h];
                if (hp.length < 0 || hp.length > kMaxHapLen) return fail(ctx, GHMM_ERR_ARG, "haplotype length out of range");
                if (hp.length > 0 && !hp.bases) return fail(ctx, GHMM_ERR_ARG, "NULL haplotype bases");
                hap_off[(size_t)hi + 1] = hap_off[(size_t)hi] + hp.length;
            }
        }
    }
    for (int64_t g = 0; g < G; g++)
        oo[(size_t)g + 1] = oo[(size_t)g] + (rro[(size_t)g + 1] - rro[(size_t)g]) * (rho[(size_t)g + 1] - rho[(size_t)g]);
    b.n_regions = G;
    b.n_reads = rro[(size_t)G];
    b.n_haps = rho[(size_t)G];
    b.read_bytes = read_off.back();
    b.hap_bytes = hap_off.back();
    b.n_out = oo[(size_t)G];
    return GHMM_OK;
}

}  // namespace

// -------------------------------------------------------------------------------------------------
// Marshal inputs into the batch's pinned staging and build tasks.
static int batch_marshal(ghmm_ctx *ctx, const Source &src, ghmm_batch &b) {
    NvtxRange range("ghmm marshal");
    const auto t_start = std::chrono::steady_clock::now();
    std::vector<int64_t> read_off, hap_off, rro, rho, oo;
    int rc = plan_sizes(ctx, src, b, read_off, hap_off, rro, rho, oo);
    if (rc) return rc;
    const int64_t G = b.n_regions, NR = b.n_reads, NH = b.n_haps;
    const int threads = hw_threads(ctx->max_threads);

    GHMM_CUDA(b.h_planes.reserve((size_t)b.read_bytes * 5), "pinned read planes");
    GHMM_CUDA(b.h_hap.reserve((size_t)b.hap_bytes * 2 + 2 * kCodePad), "pinned haplotypes");
    const size_t n_off = (size_t)(NR + 1) + (size_t)(NH + 1) + 3 * (size_t)(G + 1);
    GHMM_CUDA(b.h_off.reserve(n_off), "pinned offsets");
    GHMM_CUDA(b.h_read_region.reserve((size_t)NR), "pinned read regions");
    GHMM_CUDA(b.h_init_f.reserve((size_t)NH), "pinned init");
    GHMM_CUDA(b.h_init_d.reserve((size_t)NH), "pinned init");
    GHMM_CUDA(b.h_counters.reserve(kNumCounters + 2 * kNumBucketKeys), "pinned counters");
    GHMM_CUDA(b.h_nout.reserve(1), "pinned output count");

    uint8_t *P = b.h_planes.p;
    const int64_t RB = b.read_bytes;
    uint8_t *pb = P, *pq = P + RB, *pi = P + 2 * RB, *pd = P + 3 * RB, *pg = P + 4 * RB;
    uint8_t *hraw = b.h_hap.p, *hcode = b.h_hap.p + b.hap_bytes + kCodePad;
    memset(hcode - kCodePad, 0, kCodePad);
    memset(hcode + b.hap_bytes, 0, kCodePad);
    int64_t *o = b.h_off.p;
    std::copy(read_off.begin(), read_off.end(), o);
    std::copy(hap_off.begin(), hap_off.end(), o + NR + 1);
    std::copy(rro.begin(), rro.end(), o + NR + 1 + NH + 1);
    std::copy(rho.begin(), rho.end(), o + NR + 1 + NH + 1 + G + 1);
    std::copy(oo.begin(), oo.end(), o + NR + 1 + NH + 1 + 2 * (G + 1));

    // per-read flags: bit0 needs FP64, bit1 invalid quality.  FP64 is needed for a gap-continuation
    // penalty of 0, a non-ACGTN base, a matchToMatch probability of (almost) 0, or when the FP32 kernel's
    // rescaled insertion state could outgrow FP32 (see kernels.cu: I~ <= G * max M~ with
    // G_i = 1 + e_i G_{i-1}, and max M~ <= 2^120 / H).
    std::vector<uint8_t> read_flag((size_t)NR, 0), hap_flag((size_t)NH, 0);
    std::vector<int> region_max_read((size_t)G, 0);
    const HostTables &HT = *ctx->host_tables;

    parallel_for(G, threads, [&](int64_t g) {
        int64_t r = rro[(size_t)g];
        int mx = 0;
        int64_t hmin = INT64_MAX;
        for (int64_t h = rho[(size_t)g]; h < rho[(size_t)g + 1]; h++)
            hmin = std::min<int64_t>(hmin, hap_off[(size_t)h + 1] - hap_off[(size_t)h]);
        const double max_i_scaled = 1e37 * (double)std::max<int64_t>(hmin, 1) / std::ldexp(1.0, 120);
        for (int64_t k = 0; r < rro[(size_t)g + 1]; r++, k++) {
            const int64_t ofs = read_off[(size_t)r];
            const int R = (int)(read_off[(size_t)r + 1] - ofs);
            mx = std::max(mx, R);
            const uint8_t *sb, *sq, *si, *sd, *sg;
            if (src.flat) {
                const ghmm_flat *f = src.flat;
                const int64_t so = f->read_off[f->region_read_off[0] + r];
                sb = f->bases + so; sq = f->quals + so; si = f->ins_gop + so; sd = f->del_gop + so; sg = f->gcp + so;
            } else {
                const ghmm_read &rd = src.regions[g].reads[k];
                sb = rd.bases; sq = rd.quals; si = rd.ins_gop; sd = rd.del_gop; sg = rd.gcp;
            }
            if (R > 0) {
                memcpy(pb + ofs, sb, (size_t)R);
                memcpy(pq + ofs, sq, (size_t)R);
                memcpy(pi + ofs, si, (size_t)R);
                memcpy(pd + ofs, sd, (size_t)R);
                memcpy(pg + ofs, sg, (size_t)R);
            }
            uint8_t fl = (R == 0) ? 1 : 0;
            double growth = 1.0, expect = 0.0;
            for (int i = 0; i < R; i++) {
                expect += ctx->expect_log10_prior[sq[i]];
                if (sq[i] > kMaxQual || si[i] > 127 || sd[i] > 127 || sg[i] > 127) {
                    fl |= 2;
                    break;
                }
                if (sg[i] == 0 || base_code(sb[i]) == 0) fl |= 1;
                if (src.bound) continue;  // the gap planes are rewritten on the device
                const double mm = HT.m2m[si[i] * 128 + sd[i]];
                if (mm < 1e-6) fl |= 1 | 4;  // exact FP64 tier only (the rescaled forms divide by MM)
                if (i > 0) {
                    const double e = HT.err[sg[i]] * HT.err[si[i - 1]] /
                                     (HT.err[si[i]] * std::max(HT.m2m[si[i - 1] * 128 + sd[i - 1]], 1e-300));
                    growth = 1.0 + e * growth;
                    if (growth > max_i_scaled) fl |= 1;
                    if (growth > kMaxGrowth64) fl |= 1 | 4;  // the rescaled FP64 tier's headroom is 2^60
                }
            }
            if (src.bound) fl |= src.bound->force;
            if (expect < (double)ctx->route_fp64_log10) fl |= 1;  // predicted to underflow the FP32 pass
            read_flag[(size_t)r] = fl;
            b.h_read_region.p[r] = (int32_t)g;
        }
        region_max_read[(size_t)g] = mx;
        for (int64_t h = rho[(size_t)g]; h < rho[(size_t)g + 1]; h++) {
            const int64_t ofs = hap_off[(size_t)h];
            const int H = (int)(hap_off[(size_t)h + 1] - ofs);
            const uint8_t *sh;
            if (src.flat) {
                const ghmm_flat *f = src.flat;
                sh = f->hap_bases + f->hap_off[f->region_hap_off[0] + h];
            } else {
                sh = src.regions[g].haps[h - rho[(size_t)g]].bases;
            }
            if (H > 0) memcpy(hraw + ofs, sh, (size_t)H);
            uint8_t fl = (H == 0) ? 1 : 0;
            for (int j = 0; j < H; j++) {
                const uint8_t m = base_code(sh[j]);
                if (m == 0) fl |= 1;
                uint8_t c = base_index(sh[j]);
                if (j == 0) c |= kColFirst;
                if (j == H - 1) c |= kColLast;
                hcode[ofs + j] = c;
            }
            hap_flag[(size_t)h] = fl;
            b.h_init_f.p[h] = (float)(std::ldexp(1.0, 120) / (double)H);
            b.h_init_d.p[h] = std::ldexp(1.0, 1020) / (double)H;
        }
    });
    for (int64_t r = 0; r < NR; r++)
        if (read_flag[(size_t)r] & 2)
            return fail(ctx, GHMM_ERR_ARG,
                        "quality out of range (base quality must be <= 254; insertion, deletion and gap "
                        "continuation penalties must be 0..127)");
    b.region_max_read = region_max_read;
    b.read_exact.assign((size_t)NR, 0);
    for (int64_t r = 0; r < NR; r++) b.read_exact[(size_t)r] = (read_flag[(size_t)r] & 4) ? 1 : 0;
    b.n_direct_fp64mode = b.n_fp64mode_exact = -1;  // FP64-mode lists are built on first use
    b.max_read_len = 0;
    b.max_hap_len = 0;
    b.n_cells = 0;
    for (int64_t g = 0; g < G; g++) {
        b.max_read_len = std::max(b.max_read_len, region_max_read[(size_t)g]);
        int64_t sr = read_off[(size_t)rro[(size_t)g + 1]] - read_off[(size_t)rro[(size_t)g]];
        int64_t sh = hap_off[(size_t)rho[(size_t)g + 1]] - hap_off[(size_t)rho[(size_t)g]];
        b.n_cells += sr * sh;
    }
    for (int64_t h = 0; h < NH; h++) b.max_hap_len = std::max<int>(b.max_hap_len, (int)(hap_off[(size_t)h + 1] - hap_off[(size_t)h]));

    // ---- tasks ----
    // FP32 reads are bucketed by rows per lane K = ceil(R/32) (single strip) or K = 8 with
    // ceil(R/256) strips, paired within a region and bucket, and split into haplotype chunks.  Regions are
    // processed in parallel in contiguous parts whose outputs are concatenated in region order, so the
    // task list is the same for any thread count.
    const auto t_tasks = std::chrono::steady_clock::now();
    struct PartOut {
        std::vector<F32Task> tasks[kNumBucketKeys];
        std::vector<int64_t> cost[kNumBucketKeys];
        std::vector<PairRef> direct, direct_exact;
        int64_t max_multi_cols = 0, cells_direct = 0;
    };
    const int64_t n_parts = std::max<int64_t>(1, std::min<int64_t>(G, (int64_t)threads * 4));
    std::vector<PartOut> parts((size_t)n_parts);
    const int max_k = ctx->max_k, max_k_multi = ctx->max_k_multi;
    const int64_t chunk_cols = ctx->chunk_cols;
    parallel_for(n_parts, threads, [&](int64_t part) {
        PartOut &po = parts[(size_t)part];
        std::vector<std::pair<int64_t, int64_t>> groups;  // ((key, strips, length), read)
        std::vector<std::pair<int64_t, int64_t>> chunks;  // haplotype ranges of one task
        for (int64_t g = G * part / n_parts; g < G * (part + 1) / n_parts; g++) {
            const int64_t h0 = rho[(size_t)g], h1 = rho[(size_t)g + 1];
            const int64_t r0 = rro[(size_t)g], r1 = rro[(size_t)g + 1];
            if (h1 == h0 || r1 == r0) continue;
            bool region_fp64 = false;
            for (int64_t h = h0; h < h1; h++) region_fp64 |= (hap_flag[(size_t)h] != 0);
            const int64_t region_cols = hap_off[(size_t)h1] - hap_off[(size_t)h0];
            groups.clear();
            for (int64_t r = r0; r < r1; r++) {
                const int R = (int)(read_off[(size_t)r + 1] - read_off[(size_t)r]);
                if (region_fp64 || (read_flag[(size_t)r] & 1)) {
                    auto &dst = (read_flag[(size_t)r] & 4) ? po.direct_exact : po.direct;
                    for (int64_t h = h0; h < h1; h++) dst.push_back(PairRef{(int32_t)r, (int32_t)h});
                    po.cells_direct += (int64_t)R * region_cols;
                    continue;
                }
                // rows of the layout: the read plus its two accumulator rows (kernels.cu); at least 2 rows per lane,
                // since the accumulator rows must share lane 31
                const int rows = R + kAccRows;
                int key, ns = 1;
                if (rows <= 32 * max_k) {
                    key = std::max(2, (rows + 31) / 32);
                } else {  // fewest strips of at most max_k_multi rows per lane, then the fewest rows per lane
                    ns = (rows + 32 * max_k_multi - 1) / (32 * max_k_multi);
                    key = std::max(2, (rows + 32 * ns - 1) / (32 * ns)) | 16;
                }
                // reads are paired only within one (rows per lane, strip count) class
                groups.emplace_back(((int64_t)key * 4096 + ns) * 100000 + R, r);
            }
            std::sort(groups.begin(), groups.end());
            chunks.clear();
            for (int64_t a = h0; a < h1;) {
                int64_t e = a + 1, cols = hap_off[(size_t)a + 1] - hap_off[(size_t)a];
                while (e < h1 && cols + (hap_off[(size_t)e + 1] - hap_off[(size_t)e]) <= chunk_cols) {
                    cols += hap_off[(size_t)e + 1] - hap_off[(size_t)e];
                    e++;
                }
                chunks.emplace_back(a, e);
                a = e;
            }
            for (size_t i = 0; i < groups.size();) {
                const int64_t cls = groups[i].first / 100000;
                const int key = (int)(cls / 4096);
                const int64_t ra = groups[i].second;
                int64_t rb = -1;
                if (i + 1 < groups.size() && groups[i + 1].first / 100000 == cls) rb = groups[i + 1].second;
                i += (rb >= 0) ? 2 : 1;
                const int K = key & 15;
                const bool multi = (key & 16) != 0;
                const int S = 32 * K;
                const int Ra = (int)(read_off[(size_t)ra + 1] - read_off[(size_t)ra]);
                const int Rb = rb >= 0 ? (int)(read_off[(size_t)rb + 1] - read_off[(size_t)rb]) : 0;
                const int nstrips = multi ? (std::max(Ra, Rb) + kAccRows + S - 1) / S : 1;
                for (auto &ch : chunks) {
                    F32Task t;
                    t.read_a = (int32_t)ra;
                    t.read_b = (int32_t)rb;
                    t.hap_begin = (int32_t)ch.first;
                    t.hap_end = (int32_t)ch.second;
                    t.region = (int32_t)g;
                    t.nstrips = (int16_t)nstrips;
                    t.k = (int16_t)K;
                    t.pad_a = nstrips * S - Ra - kAccRows;
                    t.pad_b = rb >= 0 ? nstrips * S - Rb - kAccRows : nstrips * S;
                    const int64_t cols = hap_off[(size_t)ch.second] - hap_off[(size_t)ch.first];
                    if (multi) po.max_multi_cols = std::max(po.max_multi_cols, cols);
                    po.tasks[key].push_back(t);
                    po.cost[key].push_back((cols + 31) * K * nstrips);
                }
            }
        }
    }, 1);
    // buckets in key order, each ordered longest task first (ties keep region order)
    b.buckets.clear();
    int64_t total_tasks = 0, max_multi_cols = 0, n_direct = 0, n_direct_exact = 0;
    b.cells_direct = 0;
    std::vector<int64_t> bucket_pos(kNumBucketKeys + 1, 0);
    for (int key = 0; key < kNumBucketKeys; key++) {
        int64_t n = 0;
        for (auto &po : parts) n += (int64_t)po.tasks[key].size();
        bucket_pos[(size_t)key + 1] = bucket_pos[(size_t)key] + n;
    }
    for (auto &po : parts) {
        max_multi_cols = std::max(max_multi_cols, po.max_multi_cols);
        n_direct += (int64_t)po.direct.size();
        n_direct_exact += (int64_t)po.direct_exact.size();
        b.cells_direct += po.cells_direct;
    }
    total_tasks = bucket_pos[kNumBucketKeys];
    GHMM_CUDA(b.h_tasks.reserve((size_t)std::max<int64_t>(total_tasks, 1)), "pinned tasks");
    parallel_for(kNumBucketKeys, threads, [&](int64_t key) {
        const int64_t n = bucket_pos[(size_t)key + 1] - bucket_pos[(size_t)key];
        if (n == 0) return;
        std::vector<std::pair<int64_t, int64_t>> order;  // (-cost, position in region order)
        order.reserve((size_t)n);
        std::vector<const F32Task *> src_task;
        src_task.reserve((size_t)n);
        for (auto &po : parts)
            for (size_t i = 0; i < po.tasks[key].size(); i++) {
                order.emplace_back(-po.cost[key][i], (int64_t)src_task.size());
                src_task.push_back(&po.tasks[key][i]);
            }
        std::sort(order.begin(), order.end());
        F32Task *dst = b.h_tasks.p + bucket_pos[(size_t)key];
        for (int64_t i = 0; i < n; i++) dst[i] = *src_task[(size_t)order[(size_t)i].second];
    }, 1);
    for (int key = 1; key < kNumBucketKeys; key++) {
        const int64_t n = bucket_pos[(size_t)key + 1] - bucket_pos[(size_t)key];
        if (n == 0) continue;
        int bpsm = 0;
        if (fp32_kernel_occupancy(key, kBlock, &bpsm) != 0 || bpsm <= 0) bpsm = 1;
        const int64_t want = (n + kWarpsPerBlock - 1) / kWarpsPerBlock;
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->sm_count * bpsm));
        b.buckets.push_back(Bucket{key, (int)bucket_pos[(size_t)key], (int)n, grid});
    }
    b.n_tasks = total_tasks;
    b.n_direct = n_direct;
    b.n_direct_exact = n_direct_exact;
    GHMM_CUDA(b.h_direct.reserve((size_t)std::max<int64_t>(n_direct + n_direct_exact, 1)), "pinned direct pairs");
    {
        int64_t k = 0;
        for (auto &po : parts) {
            if (!po.direct.empty()) memcpy(b.h_direct.p + k, po.direct.data(), po.direct.size() * sizeof(PairRef));
            k += (int64_t)po.direct.size();
        }
        for (auto &po : parts) {
            if (!po.direct_exact.empty())
                memcpy(b.h_direct.p + k, po.direct_exact.data(), po.direct_exact.size() * sizeof(PairRef));
            k += (int64_t)po.direct_exact.size();
        }
    }
    b.scratch32_cols = max_multi_cols;
    int bpsm64 = 0;
    if (fp64_kernel_occupancy(kBlock, &bpsm64) != 0 || bpsm64 <= 0) bpsm64 = 1;
    b.fp64_grid = ctx->sm_count * bpsm64;
    b.uploaded = false;
    const auto t_end = std::chrono::steady_clock::now();
    b.ms_host_copy = std::chrono::duration<double, std::milli>(t_tasks - t_start).count();
    b.ms_host_tasks = std::chrono::duration<double, std::milli>(t_end - t_tasks).count();
    return GHMM_OK;
}

// Allocate device buffers and upload the staged batch.
static int batch_upload(ghmm_ctx *ctx, ghmm_batch &b, cudaStream_t s) {
    NvtxRange range("ghmm upload");
    const int64_t NR = b.n_reads, NH = b.n_haps, G = b.n_regions;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    GHMM_CUDA(b.d_planes.reserve((size_t)b.read_bytes * 5), "device read planes");
    GHMM_CUDA(b.d_hap.reserve((size_t)b.hap_bytes * 2 + 2 * kCodePad), "device haplotypes");
    const size_t n_off = (size_t)(NR + 1) + (size_t)(NH + 1) + 3 * (size_t)(G + 1);
    GHMM_CUDA(b.d_off.reserve(n_off), "device offsets");
    GHMM_CUDA(b.d_read_region.reserve((size_t)NR), "device read regions");
    GHMM_CUDA(b.d_init_f.reserve((size_t)NH), "device init");
    GHMM_CUDA(b.d_init_d.reserve((size_t)NH), "device init");
    GHMM_CUDA(b.d_tasks.reserve((size_t)b.n_tasks), "device tasks");
    const int64_t capacity = std::max<int64_t>(b.n_out, 1);
    GHMM_CUDA(b.d_rerun.reserve((size_t)capacity * 2), "device FP64 queues");
    GHMM_CUDA(b.d_out.reserve((size_t)std::max<int64_t>(b.n_out, 1)), "device output");
    GHMM_CUDA(b.d_counters.reserve(kNumCounters + 2 * kNumBucketKeys), "device counters");
    GHMM_CUDA(b.d_nout.reserve(1), "device output count");
    int max_grid_multi = 0;
    for (auto &bk : b.buckets)
        if (bk.key & 16) max_grid_multi = std::max(max_grid_multi, bk.grid);
    const size_t s32 = (size_t)max_grid_multi * kWarpsPerBlock * (size_t)b.scratch32_cols * 3;
    GHMM_CUDA(b.d_scratch32.reserve(std::max<size_t>(s32, 1)), "device FP32 strip scratch");
    const size_t s64 = (size_t)b.fp64_grid * kWarpsPerBlock * (size_t)std::max(b.max_hap_len, 1) * 3;
    GHMM_CUDA(b.d_scratch64.reserve(s64), "device FP64 strip scratch");

    GHMM_CUDA(cudaMemcpyAsync(b.d_planes.p, b.h_planes.p, (size_t)b.read_bytes * 5, cudaMemcpyHostToDevice, s), "H2D planes");
    GHMM_CUDA(cudaMemcpyAsync(b.d_hap.p, b.h_hap.p, (size_t)b.hap_bytes * 2 + 2 * kCodePad, cudaMemcpyHostToDevice, s),
              "H2D haplotypes");
    GHMM_CUDA(cudaMemcpyAsync(b.d_off.p, b.h_off.p, n_off * sizeof(int64_t), cudaMemcpyHostToDevice, s), "H2D offsets");
    if (NR) GHMM_CUDA(cudaMemcpyAsync(b.d_read_region.p, b.h_read_region.p, (size_t)NR * 4, cudaMemcpyHostToDevice, s), "H2D regions");
    if (NH) {
        GHMM_CUDA(cudaMemcpyAsync(b.d_init_f.p, b.h_init_f.p, (size_t)NH * 4, cudaMemcpyHostToDevice, s), "H2D init");
        GHMM_CUDA(cudaMemcpyAsync(b.d_init_d.p, b.h_init_d.p, (size_t)NH * 8, cudaMemcpyHostToDevice, s), "H2D init");
    }
    if (b.n_tasks)
        GHMM_CUDA(cudaMemcpyAsync(b.d_tasks.p, b.h_tasks.p, (size_t)b.n_tasks * sizeof(F32Task), cudaMemcpyHostToDevice, s), "H2D tasks");

    b.upload_bytes = b.read_bytes * 5 + b.hap_bytes * 2 + 2 * kCodePad + (int64_t)n_off * 8 + NR * 4 + NH * 12 +
                     b.n_tasks * (int64_t)sizeof(F32Task);
    DevBatch &d = b.dev;
    const int64_t RB = b.read_bytes;
    d.bases = b.d_planes.p;
    d.quals = b.d_planes.p + RB;
    d.ins = b.d_planes.p + 2 * RB;
    d.dels = b.d_planes.p + 3 * RB;
    d.gcp = b.d_planes.p + 4 * RB;
    d.read_off = b.d_off.p;
    d.hap_bases = b.d_hap.p;
    d.hap_code = b.d_hap.p + b.hap_bytes + kCodePad;
    d.hap_off = b.d_off.p + NR + 1;
    d.hap_init_f = b.d_init_f.p;
    d.hap_init_d = b.d_init_d.p;
    d.region_read_off = b.d_off.p + NR + 1 + NH + 1;
    d.region_hap_off = d.region_read_off + G + 1;
    d.out_off = d.region_hap_off + G + 1;
    d.read_region = b.d_read_region.p;
    d.out = b.d_out.p;
    d.tasks = b.d_tasks.p;
    d.rerun = b.d_rerun.p;
    d.counters = b.d_counters.p;
    d.bucket_info = b.d_counters.p + kNumCounters;
    d.n_out_dev = b.d_nout.p;
    d.rerun_capacity = capacity;
    d.force_rerun_every = ctx->debug_force_rerun;
    d.scratch32 = b.d_scratch32.p;
    d.scratch32_cols = b.scratch32_cols;
    d.scratch64 = b.d_scratch64.p;
    d.scratch64_cols = std::max(b.max_hap_len, 1);
    b.uploaded = true;
    return GHMM_OK;
}

// FP64 mode: every (read, hap) pair of every region, read-major; reads marked exact-only go to the exact tier.
static int fill_fp64_all(ghmm_ctx *ctx, ghmm_batch &b) {
    GHMM_CUDA(b.h_fp64all.reserve((size_t)std::max<int64_t>(b.n_out, 1)), "pinned FP64 pairs");
    const int64_t *o = b.h_off.p;
    const int64_t NR = b.n_reads, NH = b.n_haps, G = b.n_regions;
    const int64_t *rro = o + NR + 1 + NH + 1, *rho = rro + G + 1;
    int64_t k = 0;
    for (int pass = 0; pass < 2; pass++)
        for (int64_t g = 0; g < G; g++)
            for (int64_t r = rro[g]; r < rro[g + 1]; r++) {
                if ((b.read_exact[(size_t)r] != 0) != (pass == 1)) continue;
                for (int64_t h = rho[g]; h < rho[g + 1]; h++) b.h_fp64all.p[k++] = PairRef{(int32_t)r, (int32_t)h};
            }
    int64_t n_exact = 0;
    for (int64_t g = 0; g < G; g++)
        for (int64_t r = rro[g]; r < rro[g + 1]; r++)
            if (b.read_exact[(size_t)r]) n_exact += rho[g + 1] - rho[g];
    b.n_fp64mode_exact = n_exact;
    b.n_direct_fp64mode = k - n_exact;
    return GHMM_OK;
}

static int batch_enqueue(ghmm_ctx *ctx, ghmm_batch &b, int mode, cudaStream_t s);
static int batch_finish(ghmm_ctx *ctx, ghmm_batch &b);

static int batch_forward_pd(ghmm_ctx *ctx, ghmm_batch &b, bool fp32);

static int batch_forward(ghmm_ctx *ctx, ghmm_batch &b, int mode) {
    if (!b.uploaded) return fail(ctx, GHMM_ERR_STATE, "batch not uploaded");
    const bool pd_mode = mode == GHMM_MODE_PD || mode == GHMM_MODE_PD_FP32;
    if (b.has_pd != pd_mode)
        return fail(ctx, GHMM_ERR_ARG, b.has_pd ? "a PD-HMM batch runs in GHMM_MODE_PD or GHMM_MODE_PD_FP32 only"
                                                : "the PD-HMM modes need a batch from ghmm_pd_batch_create");
    if (pd_mode) return batch_forward_pd(ctx, b, mode == GHMM_MODE_PD_FP32);
    if (ctx->double_precision && mode == GHMM_MODE_FP32_RERUN) mode = GHMM_MODE_FP64;
    cudaStream_t s = ctx->stream;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    b.last_mode = mode;
    b.last_launches = 0;
    b.ms_fp32 = b.ms_fp64 = b.ms_plain = b.ms_total = 0;
    cudaEvent_t *ev = ctx->ev;
    GHMM_CUDA(cudaEventRecord(ev[0], s), "event");
    b.forward_h2d = b.forward_d2h = 0;
    if (mode == GHMM_MODE_PLAIN_FP64) {
        if (b.max_read_len > kPlainMaxRead)
            return fail(ctx, GHMM_ERR_ARG, "the plain FP64 kernel supports reads up to 2048 bases");
        const int64_t *o = b.h_off.p;
        const int64_t *rro = o + b.n_reads + 1 + b.n_haps + 1, *rho = rro + b.n_regions + 1;
        for (int64_t g = 0; g < b.n_regions; g++) {
            const int nr = (int)(rro[g + 1] - rro[g]), nh = (int)(rho[g + 1] - rho[g]);
            if (nr == 0 || nh == 0) continue;
            int e = launch_plain_region(ctx->tables, b.dev, (int)g, nr, nh, b.region_max_read[(size_t)g], s);
            if (e) return cuda_fail(ctx, (cudaError_t)e, "plain FP64 launch");
            b.last_launches++;
        }
        GHMM_CUDA(cudaEventRecord(ev[1], s), "event");
        GHMM_CUDA(cudaEventSynchronize(ev[1]), "plain FP64 kernels");
        float ms = 0;
        cudaEventElapsedTime(&ms, ev[0], ev[1]);
        b.ms_plain = b.ms_total = ms;
        b.last_rerun = 0;
        return GHMM_OK;
    }
    int rc = batch_enqueue(ctx, b, mode, s);
    if (rc) return rc;
    return batch_finish(ctx, b);
}

// The kernel sequence of one forward in two phases: 0 = FP32 buckets and the FP64 log10 epilogue, 1 = the FP64
// queue (pre-queued pairs and FP32 underflows).  Their launch arguments depend only on the batch's device
// pointers, so each phase is captured once into a CUDA graph and replayed while those stay the same; events
// recorded between the two graph launches time the phases.
static int batch_phase(ghmm_ctx *ctx, ghmm_batch &b, int phase, cudaStream_t s) {
    if (phase == 0) {
        for (auto &bk : b.buckets) {
            int e = launch_fp32_bucket(ctx->tables, b.dev, bk.key, bk.grid, kBlock, s);
            if (e) return cuda_fail(ctx, (cudaError_t)e, "FP32 bucket launch");
        }
        if (b.n_tasks > 0) {
            int e = launch_finalize_fp32(b.dev.out, b.dev.n_out_dev, ctx->sm_count, s);
            if (e) return cuda_fail(ctx, (cudaError_t)e, "FP32 finalize launch");
        }
        return GHMM_OK;
    }
    int e = launch_fp64_queue(ctx->tables, b.dev, b.fp64_grid, kBlock, s);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "FP64 queue launch");
    return GHMM_OK;
}

static int capture_phase(ghmm_ctx *ctx, ghmm_batch &b, int phase, cudaStream_t s, cudaGraphExec_t *out) {
    GHMM_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal), "graph capture");
    int rc = batch_phase(ctx, b, phase, s);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(s, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph capture");
    e = cudaGraphInstantiate(out, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "graph instantiate");
    return GHMM_OK;
}

static int kernel_launch_count(const ghmm_batch &b, int mode) {
    int n = 1;
    if (mode == GHMM_MODE_FP32_RERUN) n += (int)b.buckets.size() + (b.n_tasks > 0 ? 1 : 0);
    return n;
}

// Enqueue a forward on stream s without waiting: control words, FP64 pre-queue, the kernel graph, and the
// D2H of the counters.  batch_finish waits and reads the outcome.
static int batch_enqueue(ghmm_ctx *ctx, ghmm_batch &b, int mode, cudaStream_t s) {
    NvtxRange range("ghmm forward launch");
    if (!b.events_ready) {
        for (auto &e : b.ev) GHMM_CUDA(cudaEventCreate(&e), "cudaEventCreate");
        b.events_ready = true;
    }
    GHMM_CUDA(cudaEventRecord(b.ev[0], s), "event");
    // pre-queued pairs: queue 1 (rescaled FP64 tier) at d_rerun[0..), queue 2 (exact tier) at d_rerun[cap..)
    int64_t n_pre = b.n_direct, n_pre_exact = b.n_direct_exact;
    const PairRef *pre = b.h_direct.p;
    if (mode == GHMM_MODE_FP64) {
        if (b.n_direct_fp64mode < 0) {
            int rc = fill_fp64_all(ctx, b);
            if (rc) return rc;
        }
        n_pre = b.n_direct_fp64mode;
        n_pre_exact = b.n_fp64mode_exact;
        pre = b.h_fp64all.p;
    }
    const int64_t cap = b.dev.rerun_capacity;
    if (n_pre > 0)
        GHMM_CUDA(cudaMemcpyAsync(b.d_rerun.p, pre, (size_t)n_pre * sizeof(PairRef), cudaMemcpyHostToDevice, s),
                  "H2D FP64 pairs");
    if (n_pre_exact > 0)
        GHMM_CUDA(cudaMemcpyAsync(b.d_rerun.p + cap, pre + n_pre, (size_t)n_pre_exact * sizeof(PairRef),
                                  cudaMemcpyHostToDevice, s), "H2D exact FP64 pairs");
    int32_t *hc = b.h_counters.p;
    for (int i = 0; i < kNumCounters + 2 * kNumBucketKeys; i++) hc[i] = 0;
    hc[1] = (int32_t)n_pre;
    hc[4] = (int32_t)n_pre_exact;
    for (auto &bk : b.buckets) {
        hc[kNumCounters + bk.key] = bk.begin;
        hc[kNumCounters + kNumBucketKeys + bk.key] = bk.count;
    }
    b.h_nout.p[0] = b.n_out;
    GHMM_CUDA(cudaMemcpyAsync(b.d_counters.p, hc, (kNumCounters + 2 * kNumBucketKeys) * sizeof(int32_t),
                              cudaMemcpyHostToDevice, s), "H2D counters");
    GHMM_CUDA(cudaMemcpyAsync(b.d_nout.p, b.h_nout.p, sizeof(int64_t), cudaMemcpyHostToDevice, s), "H2D output count");
    b.forward_h2d = (n_pre + n_pre_exact) * (int64_t)sizeof(PairRef) + (kNumCounters + 2 * kNumBucketKeys) * 4 + 8;
    b.forward_d2h = kNumCounters * 4;
    // the graph signature: everything the captured launches depend on
    std::vector<unsigned char> sig(sizeof(DevBatch) + 2 * sizeof(int));
    memcpy(sig.data(), &b.dev, sizeof(DevBatch));
    memcpy(sig.data() + sizeof(DevBatch), &mode, sizeof(int));
    const int has_tasks = b.n_tasks > 0;
    memcpy(sig.data() + sizeof(DevBatch) + sizeof(int), &has_tasks, sizeof(int));
    for (auto &bk : b.buckets) {
        const int kg[2] = {bk.key, bk.grid};
        const unsigned char *k = (const unsigned char *)kg;
        sig.insert(sig.end(), k, k + sizeof(kg));
    }
    if (sig != b.graph_sig) {
        for (auto &g : b.graph) {
            if (g) cudaGraphExecDestroy(g);
            g = nullptr;
        }
        b.graph_sig.clear();
        if (mode == GHMM_MODE_FP32_RERUN && (b.n_tasks > 0 || !b.buckets.empty())) {
            int rc = capture_phase(ctx, b, 0, s, &b.graph[0]);
            if (rc) return rc;
        }
        int rc = capture_phase(ctx, b, 1, s, &b.graph[1]);
        if (rc) return rc;
        b.graph_sig = sig;
    }
    GHMM_CUDA(cudaEventRecord(b.ev[1], s), "event");
    if (b.graph[0]) GHMM_CUDA(cudaGraphLaunch(b.graph[0], s), "graph launch");
    GHMM_CUDA(cudaEventRecord(b.ev[2], s), "event");
    GHMM_CUDA(cudaGraphLaunch(b.graph[1], s), "graph launch");
    GHMM_CUDA(cudaEventRecord(b.ev[3], s), "event");
    GHMM_CUDA(cudaMemcpyAsync(hc, b.d_counters.p, kNumCounters * sizeof(int32_t), cudaMemcpyDeviceToHost, s), "D2H counters");
    GHMM_CUDA(cudaEventRecord(b.ev[4], s), "event");
    b.pending_n_pre = n_pre;
    b.pending_mode = mode;
    b.last_mode = mode;
    b.last_launches = kernel_launch_count(b, mode);
    return GHMM_OK;
}

static int batch_finish(ghmm_ctx *ctx, ghmm_batch &b) {
    NvtxRange range("ghmm forward wait");
    GHMM_CUDA(cudaEventSynchronize(b.ev[4]), "forward kernels");
    float ms = 0;
    cudaEventElapsedTime(&ms, b.ev[1], b.ev[2]);
    b.ms_fp32 = ms;
    cudaEventElapsedTime(&ms, b.ev[2], b.ev[3]);
    b.ms_fp64 = ms;
    cudaEventElapsedTime(&ms, b.ev[0], b.ev[3]);
    b.ms_total = ms;
    b.ms_plain = 0;
    const int32_t *hc = b.h_counters.p;
    if (hc[3] != 0) return fail(ctx, GHMM_ERR_CUDA, "device-side queue overflow or scratch bound exceeded");
    b.last_rerun = (int64_t)hc[1] - b.pending_n_pre;
    b.last_exact = (int64_t)hc[4];
    return GHMM_OK;
}

static int batch_results(ghmm_ctx *ctx, ghmm_batch &b, double *out) {
    if (b.n_out == 0) return GHMM_OK;
    if (!out) return fail(ctx, GHMM_ERR_ARG, "NULL output");
    GHMM_CUDA(cudaMemcpyAsync(out, b.d_out.p, (size_t)b.n_out * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream), "D2H results");
    b.results_d2h = b.n_out * 8;
    GHMM_CUDA(cudaStreamSynchronize(ctx->stream), "D2H results");
    for (int64_t i = 0; i < b.n_out; i++)
        if (!(out[i] <= 0.0)) {
            char msg[160];
            snprintf(msg, sizeof msg, "PairHMM log10 likelihood %g at output %lld is not a valid log10 probability", out[i],
                     (long long)i);
            return fail(ctx, GHMM_ERR_RESULT, msg);
        }
    return GHMM_OK;
}


// -------------------------------------------------------------------------------------------------
// Streaming queue: regions are pushed as they arrive and gathered into batches of about batch_cells
// cells; a worker thread marshals each full batch into one of two slots (pinned + device buffers, one
// CUDA stream each) and launches it, so the marshal of batch k+1 on the host, the upload of batch k+1
// and the kernels of batch k overlap, and the two streams fill each other's kernel tails.

struct QueueUnit {
    // an owned copy of pushed regions, in the flat layout ...
    std::vector<uint8_t> planes[5];
    std::vector<uint8_t> hap_bases;
    std::vector<int64_t> read_off{0}, hap_off{0}, region_read_off{0}, region_hap_off{0};
    // ... or a borrowed range of a synchronous call's input, which outlives the call
    bool borrowed = false;
    Source src;
    ghmm_flat flat{};
    std::vector<std::pair<double *, int64_t>> dests;  // output runs in region order
    int64_t cells = 0, n_out = 0, n_regions = 0;
    std::vector<int32_t> mapq;  // raw queues: mapping quality per read
    int32_t max_len = 0;        // raw queues: longest read

    void seal_flat() {  // point the flat view at the owned vectors
        flat = ghmm_flat{};
        flat.n_regions = n_regions;
        flat.region_read_off = region_read_off.data();
        flat.region_hap_off = region_hap_off.data();
        flat.read_off = read_off.data();
        flat.bases = planes[0].data();
        flat.quals = planes[1].data();
        flat.ins_gop = planes[2].data();
        flat.del_gop = planes[3].data();
        flat.gcp = planes[4].data();
        flat.hap_off = hap_off.data();
        flat.hap_bases = hap_bases.data();
        flat.out_off = nullptr;
        src = Source{};
        src.flat = &flat;
        src.n_regions = n_regions;
    }
    void drop_inputs() {
        for (auto &v : planes) std::vector<uint8_t>().swap(v);
        std::vector<uint8_t>().swap(hap_bases);
        std::vector<int64_t>().swap(read_off);
        std::vector<int64_t>().swap(hap_off);
        std::vector<int64_t>().swap(region_read_off);
        std::vector<int64_t>().swap(region_hap_off);
        std::vector<int32_t>().swap(mapq);
    }
};

struct ghmm_queue {
    ghmm_ctx *ctx = nullptr;
    int64_t batch_cells = 0;
    int mode = GHMM_MODE_FP32_RERUN;
    std::unique_ptr<QueueUnit> open;  // filled by push on the caller's thread
    std::mutex mu;
    std::condition_variable cv_work, cv_space, cv_done;
    std::deque<std::unique_ptr<QueueUnit>> ready;
    int64_t submitted = 0, retired = 0;
    bool stop = false;
    int error = GHMM_OK;
    std::string error_msg;
    ghmm_queue_info info{};
    std::thread worker;
    // raw queues: the read preparation of every batch (DRAGstr tables copied)
    bool raw = false;
    ghmm_read_prep prep{};
    ghmm_dragstr dragstr{};
    std::vector<double> str_tables;
    bool has_bound = false;
    RouteBound bound;
    // worker-owned
    ghmm_batch slot[2];
    cudaStream_t stream[2]{};
    std::unique_ptr<QueueUnit> inflight[2];
    int64_t inflight_seq[2]{};
    int64_t seq = 0;
};

namespace {

constexpr size_t kQueueMaxReady = 2;  // sealed batches waiting for the worker before push blocks

// Copy a finished slot's results to its destinations and check them (PairHMM.java:305-306).
int queue_deliver(ghmm_ctx *ctx, ghmm_batch &b, const QueueUnit &u, int threads) {
    const double *src = b.h_out.p;
    std::atomic<int64_t> bad{-1};
    std::vector<int64_t> base(u.dests.size() + 1, 0);
    for (size_t i = 0; i < u.dests.size(); i++) base[i + 1] = base[i] + u.dests[i].second;
    // blocks of at most 1M results, in parallel
    std::vector<std::pair<size_t, int64_t>> blocks;
    for (size_t i = 0; i < u.dests.size(); i++)
        for (int64_t a = 0; a < u.dests[i].second; a += (1 << 20)) blocks.emplace_back(i, a);
    parallel_for((int64_t)blocks.size(), threads, [&](int64_t k) {
        const size_t i = blocks[(size_t)k].first;
        const int64_t a = blocks[(size_t)k].second, e = std::min<int64_t>(u.dests[i].second, a + (1 << 20));
        const double *s = src + base[i];
        double *d = u.dests[i].first;
        for (int64_t j = a; j < e; j++) {
            const double v = s[j];
            d[j] = v;
            if (!(v <= 0.0)) {
                int64_t expect = -1;
                bad.compare_exchange_strong(expect, base[i] + j);
            }
        }
    }, 1);
    if (bad.load() >= 0) {
        char msg[160];
        snprintf(msg, sizeof msg, "PairHMM log10 likelihood %g at output %lld of a queued batch is not a valid log10 probability",
                 src[bad.load()], (long long)bad.load());
        return fail(ctx, GHMM_ERR_RESULT, msg);
    }
    return GHMM_OK;
}

}  // namespace

static int raw_prepare_device(ghmm_ctx *ctx, ghmm_batch &b, const int32_t *mapq, int32_t max_len,
                              const ghmm_read_prep *prep, cudaStream_t s);

namespace {

// Worker: marshal + upload (+ read preparation for a raw queue) + launch one unit into slot i (which is free).
int queue_launch(ghmm_queue *q, int i, QueueUnit &u) {
    ghmm_ctx *ctx = q->ctx;
    ghmm_batch &b = q->slot[i];
    if (q->raw) u.src.bound = q->has_bound ? &q->bound : nullptr;
    int rc = batch_marshal(ctx, u.src, b);
    if (rc) return rc;
    if (b.n_out != u.n_out) return fail(ctx, GHMM_ERR_STATE, "queued batch size mismatch");
    rc = batch_upload(ctx, b, q->stream[i]);
    if (rc) return rc;
    if (q->raw) {
        rc = raw_prepare_device(ctx, b, u.mapq.data(), u.max_len, &q->prep, q->stream[i]);
        if (rc) return rc;
    }
    rc = batch_enqueue(ctx, b, q->mode, q->stream[i]);
    if (rc) return rc;
    if (b.n_out > 0) {
        GHMM_CUDA(b.h_out.reserve((size_t)b.n_out), "pinned results");
        GHMM_CUDA(cudaMemcpyAsync(b.h_out.p, b.d_out.p, (size_t)b.n_out * sizeof(double), cudaMemcpyDeviceToHost,
                                  q->stream[i]), "D2H results");
        GHMM_CUDA(cudaEventRecord(b.ev[4], q->stream[i]), "event");
    }
    b.results_d2h = b.n_out * 8;
    return GHMM_OK;
}

int queue_retire(ghmm_queue *q, int i) {
    ghmm_ctx *ctx = q->ctx;
    ghmm_batch &b = q->slot[i];
    int rc = batch_finish(ctx, b);
    if (!rc) rc = queue_deliver(ctx, b, *q->inflight[i], hw_threads(ctx->max_threads));
    std::lock_guard<std::mutex> lk(q->mu);
    if (!rc) {
        ghmm_queue_info &in = q->info;
        in.n_batches++;
        in.n_launches += b.last_launches;
        in.n_rerun += b.last_mode == GHMM_MODE_FP32_RERUN ? b.last_rerun : 0;
        in.n_fp64_direct += b.last_mode == GHMM_MODE_FP64 ? b.n_out : b.n_direct + b.n_direct_exact;
        in.n_fp64_exact += b.last_exact;
        in.n_cells_fp64_direct += b.last_mode == GHMM_MODE_FP64 ? b.n_cells : b.cells_direct;
        in.h2d_bytes += b.upload_bytes + b.forward_h2d;
        in.d2h_bytes += b.forward_d2h + b.results_d2h;
        in.ms_fp32 += b.ms_fp32;
        in.ms_fp64 += b.ms_fp64;
        in.ms_host_marshal += b.ms_host_copy;
        in.ms_host_tasks += b.ms_host_tasks;
    }
    q->inflight[i].reset();
    q->retired++;
    q->cv_done.notify_all();
    return rc;
}

void queue_record_error(ghmm_queue *q, int rc, const std::string &msg) {
    std::lock_guard<std::mutex> lk(q->mu);
    if (q->error == GHMM_OK) {
        q->error = rc;
        q->error_msg = msg;
    }
}

void queue_worker(ghmm_queue *q) {
    std::string err;
    t_error_sink = &err;
    cudaSetDevice(q->ctx->device);
    for (;;) {
        std::unique_ptr<QueueUnit> u;
        int oldest = -1;
        {
            std::unique_lock<std::mutex> lk(q->mu);
            for (;;) {
                if (!q->ready.empty()) {
                    u = std::move(q->ready.front());
                    q->ready.pop_front();
                    q->cv_space.notify_all();
                    break;
                }
                oldest = -1;
                for (int i = 0; i < 2; i++)
                    if (q->inflight[i] && (oldest < 0 || q->inflight_seq[i] < q->inflight_seq[oldest])) oldest = i;
                if (oldest >= 0) {
                    // nothing to marshal: retire the oldest batch once it is done, polling so that a newly
                    // sealed batch is taken up while it runs
                    if (cudaEventQuery(q->slot[oldest].ev[4]) != cudaErrorNotReady) break;
                    q->cv_work.wait_for(lk, std::chrono::microseconds(200));
                    oldest = -1;
                    continue;
                }
                if (q->stop) return;
                q->cv_work.wait(lk);
            }
        }
        if (!u) {  // retire the oldest finished batch
            int rc = queue_retire(q, oldest);
            if (rc) queue_record_error(q, rc, err);
            continue;
        }
        int i = q->inflight[0] ? (q->inflight[1] ? -1 : 1) : 0;
        if (i < 0) {  // both busy: retire the older one and reuse its slot
            i = q->inflight_seq[0] < q->inflight_seq[1] ? 0 : 1;
            int rc = queue_retire(q, i);
            if (rc) queue_record_error(q, rc, err);
        }
        bool failed;
        {
            std::lock_guard<std::mutex> lk(q->mu);
            failed = q->error != GHMM_OK;
        }
        int rc = failed ? GHMM_OK : queue_launch(q, i, *u);
        if (failed || rc) {  // after an error the remaining batches are dropped, not computed
            if (rc) queue_record_error(q, rc, err);
            std::lock_guard<std::mutex> lk(q->mu);
            q->retired++;
            q->cv_done.notify_all();
            continue;
        }
        if (!u->borrowed) u->drop_inputs();
        q->inflight[i] = std::move(u);
        q->inflight_seq[i] = ++q->seq;
    }
}

// Hand the open unit to the worker (blocks while kQueueMaxReady units already wait).
void queue_submit(ghmm_queue *q, std::unique_ptr<QueueUnit> u) {
    if (!u->borrowed) u->seal_flat();
    std::unique_lock<std::mutex> lk(q->mu);
    q->cv_space.wait(lk, [&] { return q->ready.size() < kQueueMaxReady || q->error != GHMM_OK; });
    q->ready.push_back(std::move(u));
    q->submitted++;
    q->cv_work.notify_all();
}

int queue_wait_all(ghmm_queue *q) {
    std::unique_lock<std::mutex> lk(q->mu);
    q->cv_done.wait(lk, [&] { return q->retired == q->submitted; });
    return q->error;
}

// Make q a queue of raw reads with the (already checked) read preparation prep (DRAGstr tables copied), or, with
// prep NULL, a queue of prepared reads again.  Only while no batch is queued or in flight.
void queue_set_raw(ghmm_queue *q, const ghmm_read_prep *prep, const RouteBound *bound) {
    q->raw = prep != nullptr;
    q->has_bound = false;
    q->str_tables.clear();
    if (!prep) return;
    q->prep = *prep;
    q->prep.dragstr = nullptr;
    if (prep->dragstr) {
        const ghmm_dragstr &d = *prep->dragstr;
        const size_t cells = (size_t)d.max_period * (size_t)d.max_repeats;
        q->str_tables.assign(d.gop, d.gop + cells);
        q->str_tables.insert(q->str_tables.end(), d.gcp, d.gcp + cells);
        q->dragstr = ghmm_dragstr{d.max_period, d.max_repeats, q->str_tables.data(), q->str_tables.data() + cells};
        q->prep.dragstr = &q->dragstr;
    }
    if (bound) {
        q->has_bound = true;
        q->bound = *bound;
    }
}

// raw_prep: NULL for a queue of prepared reads; else the (already checked) read preparation of a raw queue
int queue_open(ghmm_ctx *ctx, int64_t batch_cells, ghmm_queue **out, const ghmm_read_prep *raw_prep = nullptr,
               const RouteBound *bound = nullptr) {
    auto *q = new ghmm_queue();
    q->ctx = ctx;
    q->batch_cells = batch_cells > 0 ? batch_cells : (int64_t)2e11;
    q->mode = ctx->double_precision ? GHMM_MODE_FP64 : GHMM_MODE_FP32_RERUN;
    if (raw_prep) queue_set_raw(q, raw_prep, bound);
    for (auto &st : q->stream) {
        cudaError_t e = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            for (auto &s2 : q->stream)
                if (s2) cudaStreamDestroy(s2);
            delete q;
            return cuda_fail(ctx, e, "queue stream");
        }
    }
    q->worker = std::thread(queue_worker, q);
    ctx->open_queues++;
    *out = q;
    return GHMM_OK;
}

void queue_close(ghmm_queue *q) {
    {
        std::lock_guard<std::mutex> lk(q->mu);
        q->stop = true;
        q->cv_work.notify_all();
    }
    q->worker.join();
    cudaSetDevice(q->ctx->device);
    for (int i = 0; i < 2; i++) {
        if (q->stream[i]) cudaStreamSynchronize(q->stream[i]);
        q->slot[i].release();
        if (q->stream[i]) cudaStreamDestroy(q->stream[i]);
    }
    q->ctx->open_queues--;
    delete q;
}

// The error a queue recorded, moved into the context's message on the caller's thread.
int queue_status(ghmm_queue *q) {
    std::lock_guard<std::mutex> lk(q->mu);
    if (q->error != GHMM_OK) q->ctx->last_error = q->error_msg;
    return q->error;
}

// Regions [g0, g1) of a synchronous call, borrowed.  out_base points at region g0's first result.
std::unique_ptr<QueueUnit> borrowed_unit(const Source &src, int64_t g0, int64_t g1, double *out_base, int64_t n_out,
                                         int64_t cells) {
    auto u = std::make_unique<QueueUnit>();
    u->borrowed = true;
    u->n_regions = g1 - g0;
    if (src.flat) {
        u->flat = *src.flat;
        u->flat.n_regions = g1 - g0;
        u->flat.region_read_off = src.flat->region_read_off + g0;
        u->flat.region_hap_off = src.flat->region_hap_off + g0;
        u->src.flat = &u->flat;
    } else {
        u->src.regions = src.regions + g0;
    }
    u->src.n_regions = g1 - g0;
    u->n_out = n_out;
    u->cells = cells;
    if (n_out > 0) u->dests.emplace_back(out_base, n_out);
    return u;
}

// Large synchronous inputs run as a pipeline of batches through the context's own queue: the first batch
// is small so that the GPU starts early, later ones grow to a third of the input.
constexpr int64_t kPipelineMinCells = (int64_t)6e10;

// Raw reads (mapq non-NULL, src.regions over the raw view's reads): every batch gets the read preparation prep on
// the device after its upload.
int pipelined_compute(ghmm_ctx *ctx, const Source &src, const std::vector<int64_t> &reg_cells,
                      const std::vector<int64_t> &reg_out, double *out, const int32_t *mapq = nullptr,
                      int32_t max_len = 0, const ghmm_read_prep *prep = nullptr, const RouteBound *bound = nullptr) {
    if (!ctx->pipe) {
        int rc = queue_open(ctx, 0, &ctx->pipe);
        if (rc) return rc;
    }
    ghmm_queue *q = ctx->pipe;
    {
        std::lock_guard<std::mutex> lk(q->mu);
        q->error = GHMM_OK;
        q->error_msg.clear();
        q->mode = ctx->double_precision ? GHMM_MODE_FP64 : GHMM_MODE_FP32_RERUN;
        queue_set_raw(q, mapq ? prep : nullptr, bound);
    }
    const int64_t G = src.n_regions;
    std::vector<int64_t> first_read;  // raw reads: the batch's reads' mapping qualities go with the batch
    if (mapq) {
        first_read.assign((size_t)G + 1, 0);
        for (int64_t g = 0; g < G; g++) first_read[(size_t)g + 1] = first_read[(size_t)g] + src.regions[g].n_reads;
    }
    int64_t total = 0;
    for (int64_t g = 0; g < G; g++) total += reg_cells[(size_t)g];
    int64_t target = std::max<int64_t>(total / 16, 1), g0 = 0;
    while (g0 < G) {
        int64_t g1 = g0, c = 0;
        while (g1 < G && (c < target || g1 == g0)) c += reg_cells[(size_t)g1++];
        if (G - g1 < 8) {  // do not leave a sliver
            for (; g1 < G; g1++) c += reg_cells[(size_t)g1];
        }
        auto u = borrowed_unit(src, g0, g1, out + reg_out[(size_t)g0], reg_out[(size_t)g1] - reg_out[(size_t)g0], c);
        if (mapq) {
            u->mapq.assign(mapq + first_read[(size_t)g0], mapq + first_read[(size_t)g1]);
            u->max_len = max_len;
        }
        queue_submit(q, std::move(u));
        target = std::min(target * 5 / 2, std::max<int64_t>(total / 3, 1));
        g0 = g1;
    }
    int rc = queue_wait_all(q);
    {
        std::lock_guard<std::mutex> lk(q->mu);
        queue_set_raw(q, nullptr, nullptr);
    }
    if (rc) return queue_status(q);
    return GHMM_OK;
}

// Per-region cells and output offsets of a region array or flat input; false if a count is negative.
bool region_sizes(const Source &src, std::vector<int64_t> &cells, std::vector<int64_t> &outo) {
    const int64_t G = src.n_regions;
    cells.assign((size_t)G, 0);
    outo.assign((size_t)G + 1, 0);
    for (int64_t g = 0; g < G; g++) {
        int64_t sr = 0, sh = 0, nr, nh;
        if (src.flat) {
            const ghmm_flat *f = src.flat;
            nr = f->region_read_off[g + 1] - f->region_read_off[g];
            nh = f->region_hap_off[g + 1] - f->region_hap_off[g];
            if (nr < 0 || nh < 0) return false;
            sr = f->read_off[f->region_read_off[g + 1]] - f->read_off[f->region_read_off[g]];
            sh = f->hap_off[f->region_hap_off[g + 1]] - f->hap_off[f->region_hap_off[g]];
        } else {
            const ghmm_region &rg = src.regions[g];
            nr = rg.n_reads;
            nh = rg.n_haps;
            if (nr < 0 || nh < 0 || (nr > 0 && !rg.reads) || (nh > 0 && !rg.haps)) return false;
            for (int32_t r = 0; r < rg.n_reads; r++) sr += std::max(rg.reads[r].length, 0);
            for (int32_t h = 0; h < rg.n_haps; h++) sh += std::max(rg.haps[h].length, 0);
        }
        cells[(size_t)g] = sr * sh;
        outo[(size_t)g + 1] = outo[(size_t)g] + nr * nh;
    }
    return true;
}

// Synchronous compute of regions or flat input: one batch for small inputs, the pipeline for large ones.
int compute_sync(ghmm_ctx *ctx, const Source &src, double *out) {
    std::vector<int64_t> cells, outo;
    if (!region_sizes(src, cells, outo)) return fail(ctx, GHMM_ERR_ARG, "negative count or NULL array in a region");
    int64_t total = 0;
    for (auto c : cells) total += c;
    if (outo.back() > 0 && !out) return fail(ctx, GHMM_ERR_ARG, "NULL output");
    if (total >= kPipelineMinCells && src.n_regions >= 4) return pipelined_compute(ctx, src, cells, outo, out);
    ghmm_batch &b = ctx->scratch_batch;
    int rc = batch_marshal(ctx, src, b);
    if (!rc) rc = batch_upload(ctx, b, ctx->stream);
    if (!rc) rc = batch_forward(ctx, b, ctx->double_precision ? GHMM_MODE_FP64 : GHMM_MODE_FP32_RERUN);
    if (!rc) rc = batch_results(ctx, b, out);
    return rc;
}

}  // namespace


// -------------------------------------------------------------------------------------------------
// PD-HMM batches: the regular marshal over the haplotypes' bases, plus per haplotype column the PD flags and the
// HMM state codes (PdPlanes), and a forward that runs every pair through pd.cu.

namespace {

// State sequence along one row (LoglessPDPairHMM.java:62-142): the state a column is processed in, then AFTER_DEL
// ends, DEL_START enters INSIDE_DEL, DEL_END enters AFTER_DEL.  Returns the state after the last column.
int pd_states(const uint8_t *f, int H, int start, uint8_t *code, int shift) {
    int st = start;
    for (int j = 0; j < H; j++) {
        code[j] |= (uint8_t)(st << shift);
        if (st == 2) st = 0;
        if (f[j] & 2) st = 1;
        if (f[j] & 4) st = 2;
    }
    return st;
}

bool pd_read_base_ok(uint8_t x) {
    switch (x) {
        case 'A': case 'C': case 'G': case 'T': case 'a': case 'c': case 'g': case 't': case 'N': return true;
        default: return false;
    }
}

}  // namespace

static int pd_marshal(ghmm_ctx *ctx, const ghmm_pd_region *regs, int64_t G, ghmm_batch &b) {
    std::vector<ghmm_region> rr((size_t)G);
    std::vector<std::vector<ghmm_hap>> hh((size_t)G);
    std::vector<const uint8_t *> pdp;
    for (int64_t g = 0; g < G; g++) {
        const ghmm_pd_region &rg = regs[g];
        if (rg.n_reads < 0 || rg.n_haps < 0 || (rg.n_reads > 0 && !rg.reads) || (rg.n_haps > 0 && !rg.haps))
            return fail(ctx, GHMM_ERR_ARG, "bad PD region");
        hh[(size_t)g].resize((size_t)rg.n_haps);
        for (int32_t h = 0; h < rg.n_haps; h++) {
            const ghmm_pd_hap &hp = rg.haps[h];
            if (hp.length > 0 && (!hp.bases || !hp.pd_bases)) return fail(ctx, GHMM_ERR_ARG, "NULL PD haplotype array");
            hh[(size_t)g][(size_t)h] = ghmm_hap{hp.bases, hp.length};
            pdp.push_back(hp.pd_bases);
        }
        rr[(size_t)g] = ghmm_region{rg.reads, rg.n_reads, hh[(size_t)g].data(), rg.n_haps};
    }
    Source src;
    src.regions = rr.data();
    src.n_regions = G;
    int rc = batch_marshal(ctx, src, b);
    if (rc) return rc;
    const int64_t NH = b.n_haps, HB = b.hap_bytes;
    GHMM_CUDA(b.h_pd.reserve((size_t)std::max<int64_t>(2 * HB, 1)), "pinned PD planes");
    const int64_t *o = b.h_off.p;
    const int64_t *hap_off = o + b.n_reads + 1;
    uint8_t *flags = b.h_pd.p, *states = b.h_pd.p + HB;
    parallel_for(NH, hw_threads(ctx->max_threads), [&](int64_t h) {
        const int64_t a = hap_off[h];
        const int H = (int)(hap_off[h + 1] - a);
        if (H <= 0) return;
        memcpy(flags + a, pdp[(size_t)h], (size_t)H);
        uint8_t *code = states + a;
        memset(code, 0, (size_t)H);
        const int end1 = pd_states(flags + a, H, 0, code, 0);
        pd_states(flags + a, H, end1, code, 2);
        for (int j = 0; j < H; j++)
            if (flags[a + j] & 4) code[j] |= 16;
    });
    // a read base outside ACGTacgtN that meets an undetermined SNP column throws in the reference
    const int64_t *rro = o + b.n_reads + 1 + NH + 1, *rho = rro + G + 1;
    const uint8_t *bases = b.h_planes.p;
    const uint8_t *hraw = b.h_hap.p;
    for (int64_t g = 0; g < G; g++)
        for (int64_t r = rro[g]; r < rro[g + 1]; r++)
            for (int64_t i = o[r]; i < o[r + 1]; i++) {
                const uint8_t x = bases[i];
                if (pd_read_base_ok(x)) continue;
                for (int64_t h = rho[g]; h < rho[g + 1]; h++)
                    for (int64_t j = hap_off[h]; j < hap_off[h + 1]; j++)
                        if ((flags[j] & 1) && hraw[j] != x && hraw[j] != 'N')
                            return fail(ctx, GHMM_ERR_ARG, "Found unexpected base in alt alleles");
            }
    b.has_pd = true;
    return GHMM_OK;
}

static int pd_upload(ghmm_ctx *ctx, ghmm_batch &b, cudaStream_t s) {
    int rc = batch_upload(ctx, b, s);
    if (rc) return rc;
    const int64_t HB = b.hap_bytes;
    GHMM_CUDA(b.d_pd.reserve((size_t)std::max<int64_t>(2 * HB, 1)), "device PD planes");
    if (HB > 0)
        GHMM_CUDA(cudaMemcpyAsync(b.d_pd.p, b.h_pd.p, (size_t)(2 * HB), cudaMemcpyHostToDevice, s), "H2D PD planes");
    b.pd.flags = b.d_pd.p;
    b.pd.states = b.d_pd.p + HB;
    b.upload_bytes += 2 * HB;
    return GHMM_OK;
}

// fp32: every pair in the FP32 PD kernel, then the pairs whose sums underflow in the FP64 one (K = 4 for all);
// otherwise every pair in FP64
static int batch_forward_pd(ghmm_ctx *ctx, ghmm_batch &b, bool fp32) {
    cudaStream_t s = ctx->stream;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    // every pair, grouped by the rows per lane K of its read (the strip height 32 K, K = 1..4, that needs the
    // fewest rows; ties to the larger K, i.e. fewer strips), read-major per region within a group
    GHMM_CUDA(b.h_fp64all.reserve((size_t)std::max<int64_t>(b.n_out, 1)), "pinned PD pairs");
    const int64_t *o = b.h_off.p;
    const int64_t *rro = o + b.n_reads + 1 + b.n_haps + 1, *rho = rro + b.n_regions + 1;
    const int maxk = fp32 ? kPdMaxK32 : kPdMaxK;
    auto pick_k = [maxk](int64_t R) {
        int best_k = maxk;
        int64_t best_rows = INT64_MAX;
        for (int k = maxk; k >= 1; --k) {
            const int64_t rows = ((R + 32 * k - 1) / (32 * k)) * 32 * k;
            if (rows < best_rows) best_rows = rows, best_k = k;
        }
        return best_k;
    };
    int64_t kcount[kPdMaxK32 + 1] = {0};
    for (int64_t g = 0; g < b.n_regions; g++)
        for (int64_t r = rro[g]; r < rro[g + 1]; r++) kcount[pick_k(o[r + 1] - o[r])] += rho[g + 1] - rho[g];
    int64_t kbegin[kPdMaxK32 + 2] = {0};
    for (int kk = 1; kk <= maxk; kk++) kbegin[kk + 1] = kbegin[kk] + kcount[kk];
    int64_t kpos[kPdMaxK32 + 1];
    for (int kk = 1; kk <= maxk; kk++) kpos[kk] = kbegin[kk];
    for (int64_t g = 0; g < b.n_regions; g++)
        for (int64_t r = rro[g]; r < rro[g + 1]; r++) {
            const int kk = pick_k(o[r + 1] - o[r]);
            for (int64_t h = rho[g]; h < rho[g + 1]; h++) b.h_fp64all.p[kpos[kk]++] = PairRef{(int32_t)r, (int32_t)h};
        }
    const int64_t k = kbegin[maxk + 1];
    int bpsm = 0;
    if (pd_kernel_occupancy(&bpsm) != 0 || bpsm <= 0) bpsm = 1;
    const int grid = ctx->sm_count * bpsm;
    const size_t scr = (size_t)grid * (kBlock / 32) * (size_t)std::max(b.max_hap_len, 1) * 6;
    GHMM_CUDA(b.d_scratch64.reserve(scr), "device PD strip scratch");
    b.dev.scratch64 = b.d_scratch64.p;
    b.dev.scratch64_cols = std::max(b.max_hap_len, 1);
    if (!b.events_ready) {
        for (auto &e : b.ev) GHMM_CUDA(cudaEventCreate(&e), "cudaEventCreate");
        b.events_ready = true;
    }
    GHMM_CUDA(cudaEventRecord(b.ev[0], s), "event");
    if (k > 0)
        GHMM_CUDA(cudaMemcpyAsync(b.d_rerun.p, b.h_fp64all.p, (size_t)k * sizeof(PairRef), cudaMemcpyHostToDevice, s),
                  "H2D PD pairs");
    int32_t *hc = b.h_counters.p;
    for (int i = 0; i < kNumCounters + 2 * kNumBucketKeys; i++) hc[i] = 0;
    hc[1] = (int32_t)k;
    GHMM_CUDA(cudaMemcpyAsync(b.d_counters.p, hc, (kNumCounters + 2 * kNumBucketKeys) * sizeof(int32_t),
                              cudaMemcpyHostToDevice, s), "H2D counters");
    GHMM_CUDA(cudaEventRecord(b.ev[1], s), "event");
    int launches = 0;
    for (int kk = maxk; kk >= 1; --kk) {  // longest strips first
        if (kcount[kk] == 0) continue;
        const int cursor = (fp32 ? kCounterPdF32Base : kCounterPdBase) + kk;
        int e = launch_pd(ctx->tables, b.dev, b.pd, kk, fp32, (int)kbegin[kk], (int)kcount[kk], cursor, nullptr, grid, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "PD-HMM launch");
        launches++;
    }
    GHMM_CUDA(cudaEventRecord(b.ev[4], s), "event");
    if (fp32 && k > 0) {  // the FP32 pass's underflows, queued at rerun[capacity..), in FP64
        int e = launch_pd(ctx->tables, b.dev, b.pd, kPdMaxK, false, (int)b.dev.rerun_capacity, 0,
                          kCounterPdRerunCursor, b.d_counters.p + kCounterPdRerun, grid, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "PD-HMM FP64 rerun launch");
        launches++;
    }
    GHMM_CUDA(cudaEventRecord(b.ev[2], s), "event");
    GHMM_CUDA(cudaMemcpyAsync(hc, b.d_counters.p, kNumCounters * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
              "D2H counters");
    GHMM_CUDA(cudaEventRecord(b.ev[3], s), "event");
    GHMM_CUDA(cudaEventSynchronize(b.ev[3]), "PD-HMM kernel");
    float ms = 0, ms_a = 0, ms_b = 0;
    cudaEventElapsedTime(&ms_a, b.ev[1], b.ev[4]);
    cudaEventElapsedTime(&ms_b, b.ev[4], b.ev[2]);
    b.ms_fp32 = fp32 ? ms_a : 0;
    b.ms_fp64 = fp32 ? ms_b : ms_a + ms_b;
    b.ms_plain = 0;
    cudaEventElapsedTime(&ms, b.ev[0], b.ev[3]);
    b.ms_total = ms;
    b.last_mode = fp32 ? GHMM_MODE_PD_FP32 : GHMM_MODE_PD;
    b.last_launches = launches;
    b.last_rerun = fp32 ? hc[kCounterPdRerun] : 0;
    b.last_exact = 0;
    b.forward_h2d = k * (int64_t)sizeof(PairRef) + (kNumCounters + 2 * kNumBucketKeys) * 4;
    b.forward_d2h = kNumCounters * 4;
    if (hc[3] == 1) return fail(ctx, GHMM_ERR_CUDA, "PD-HMM FP64 rerun queue overflow");
    if (hc[3] != 0) return fail(ctx, GHMM_ERR_CUDA, "device-side scratch bound exceeded");
    return GHMM_OK;
}


// -------------------------------------------------------------------------------------------------
// Raw reads: the regular marshal over the reads' bases and raw qualities (45 where a read has no BI / BD tag, the
// constant gap continuation penalty), then prep.cu rewrites the quality planes on the device.  The host's routing
// checks see the raw qualities; a read whose prepared qualities would make the FP32 or rescaled FP64 forms
// overflow still ends up exact, because a non-finite sum sends its pair on to the next tier.

namespace {

struct RawView {
    std::vector<ghmm_region> regions;
    std::vector<ghmm_read> reads;  // every region's reads, region after region
    std::vector<uint8_t> q45, qgcp;  // shared constant planes
    std::vector<int32_t> mapq;
    int32_t max_len = 0;
    bool has_bound = false;
    RouteBound bound;
};

// Math.round(double) (half up), for table values already checked to lie in [-0.5, 127.5)
int java_round(double x) {
    double r = std::floor(x);
    if (x - r >= 0.5) r += 1.0;
    return (int)r;
}

// The penalties DRAGstr tables can impute (Math.round(min(40, gop)) and Math.round(gcp) over every cell, plus 45 / 10
// at the last base) give the routing flags of the batch.
int dragstr_bound(ghmm_ctx *ctx, const ghmm_dragstr &d, RouteBound &rb) {
    const size_t cells = (size_t)d.max_period * (size_t)d.max_repeats;
    int gmin = 45, gmax = 45, cmin = 10;
    for (size_t k = 0; k < cells; k++) {
        const double g = d.gop[k], c = d.gcp[k];
        if (!(g >= -0.5) || !(c >= -0.5 && c < 127.5))
            return fail(ctx, GHMM_ERR_ARG, "DRAGstr tables: gop >= 0 and gcp 0..127 expected");
        const int gq = java_round(std::min(40.0, g)), cq = java_round(c);
        gmin = std::min(gmin, gq);
        gmax = std::max(gmax, gq);
        cmin = std::min(cmin, cq);
    }
    const HostTables &HT = *ctx->host_tables;
    double mm_min = 1.0;
    for (int g = gmin; g <= gmax; g++) mm_min = std::min(mm_min, HT.m2m[g * 128 + g]);
    rb.force = 0;
    if (cmin == 0) rb.force |= 1;
    if (mm_min < 1e-6) rb.force |= 1 | 4;
    return GHMM_OK;
}

// Checks of one raw region and its reads shared by the raw entry points: 0, or an index into kRawErrors
const char *const kRawErrors[] = {"", "bad raw region", "read length out of range", "NULL read array",
                                  "mapping quality 0..255"};
int raw_region_problem(const ghmm_raw_region &rg, int32_t *max_len) {
    if (rg.n_reads < 0 || rg.n_haps < 0 || (rg.n_reads > 0 && !rg.reads) || (rg.n_haps > 0 && !rg.haps)) return 1;
    int32_t mx = 0;
    for (int32_t r = 0; r < rg.n_reads; r++) {
        const ghmm_raw_read &rd = rg.reads[r];
        if (rd.length < 0 || rd.length > kMaxReadLen) return 2;
        if (rd.length > 0 && (!rd.bases || !rd.quals)) return 3;
        if (rd.mapping_quality < 0 || rd.mapping_quality > 255) return 4;
        mx = std::max(mx, rd.length);
    }
    *max_len = mx;
    return 0;
}

int raw_view(ghmm_ctx *ctx, const ghmm_raw_region *raw, int64_t G, const ghmm_read_prep *prep, RawView &v) {
    if (!prep) return fail(ctx, GHMM_ERR_ARG, "NULL read preparation arguments");
    if (prep->gcp < 1 || prep->gcp > 127) return fail(ctx, GHMM_ERR_ARG, "gap continuation penalty must be 1..127");
    if (prep->base_quality_threshold < 6 || prep->base_quality_threshold > 127)
        return fail(ctx, GHMM_ERR_ARG, "base quality threshold must be 6..127 (QualityUtils.MIN_USABLE_Q_SCORE)");
    if (!(prep->pcr_rate_factor >= 0.0)) return fail(ctx, GHMM_ERR_ARG, "PCR rate factor must be >= 0");
    if (prep->dragstr) {
        const ghmm_dragstr &d = *prep->dragstr;
        if (d.max_period < 1 || d.max_period > kDragstrMaxPeriod || d.max_repeats < 1 || d.max_repeats > (1 << 16) ||
            !d.gop || !d.gcp)
            return fail(ctx, GHMM_ERR_ARG, "DRAGstr tables: max_period 1..32, max_repeats >= 1, non-NULL gop and gcp");
        const int rc = dragstr_bound(ctx, d, v.bound);
        if (rc) return rc;
        v.has_bound = true;
    }
    // checks and per-region read counts in parallel; the first bad region (in order) names the error
    const int threads = hw_threads(ctx->max_threads);
    std::vector<int8_t> bad((size_t)G, 0);
    std::vector<int32_t> region_max((size_t)G, 0);
    parallel_for(G, threads, [&](int64_t g) {
        bad[(size_t)g] = (int8_t)raw_region_problem(raw[g], &region_max[(size_t)g]);
    }, 16);
    int32_t max_len = 0;
    std::vector<int64_t> first((size_t)G + 1, 0);
    for (int64_t g = 0; g < G; g++) {
        if (bad[(size_t)g]) return fail(ctx, GHMM_ERR_ARG, kRawErrors[bad[(size_t)g]]);
        max_len = std::max(max_len, region_max[(size_t)g]);
        first[(size_t)g + 1] = first[(size_t)g] + raw[g].n_reads;
    }
    if (prep->dragstr && max_len > kDragstrMaxRead)
        return fail(ctx, GHMM_ERR_ARG, "the DRAGstr imputation takes reads of up to 28000 bases");
    v.max_len = max_len;
    v.q45.assign((size_t)std::max(max_len, 1), 45);
    v.qgcp.assign((size_t)std::max(max_len, 1), (uint8_t)prep->gcp);
    v.regions.resize((size_t)G);
    v.reads.resize((size_t)first[(size_t)G]);
    v.mapq.resize((size_t)first[(size_t)G]);
    parallel_for(G, threads, [&](int64_t g) {
        const ghmm_raw_region &rg = raw[g];
        ghmm_read *rr = v.reads.data() + first[(size_t)g];
        int32_t *mq = v.mapq.data() + first[(size_t)g];
        for (int32_t r = 0; r < rg.n_reads; r++) {
            const ghmm_raw_read &rd = rg.reads[r];
            rr[r] = ghmm_read{rd.bases, rd.quals, rd.ins_quals ? rd.ins_quals : v.q45.data(),
                              rd.del_quals ? rd.del_quals : v.q45.data(), v.qgcp.data(), rd.length};
            mq[r] = rd.mapping_quality;
        }
        v.regions[(size_t)g] = ghmm_region{rr, rg.n_reads, rg.haps, rg.n_haps};
    }, 16);
    return GHMM_OK;
}

}  // namespace

static int raw_prepare_device(ghmm_ctx *ctx, ghmm_batch &b, const int32_t *mapq, int32_t max_len,
                              const ghmm_read_prep *prep, cudaStream_t s) {
    NvtxRange range("ghmm read preparation");
    const int64_t NR = b.n_reads;
    if (NR == 0) return GHMM_OK;
    GHMM_CUDA(b.h_mapq.reserve((size_t)NR), "pinned mapping qualities");
    GHMM_CUDA(b.d_mapq.reserve((size_t)NR), "device mapping qualities");
    memcpy(b.h_mapq.p, mapq, (size_t)NR * sizeof(int32_t));
    GHMM_CUDA(cudaMemcpyAsync(b.d_mapq.p, b.h_mapq.p, (size_t)NR * sizeof(int32_t), cudaMemcpyHostToDevice, s),
              "H2D mapping qualities");
    PrepArgs p{};
    p.mapq = b.d_mapq.p;
    p.pcr = prep->pcr_rate_factor != 0.0;
    p.cap_to_mapq = prep->cap_to_mapq ? 1 : 0;
    p.threshold = prep->base_quality_threshold;
    // getErrorModelAdjustedQual (PairHMMLikelihoodCalculationEngine.java:355-358): max(10, fastRound(40 -
    // exp(repeatLength / (rateFactor pi)) + 1))
    for (int rl = 0; rl <= 20; rl++) {
        double d = 40.0;
        if (p.pcr) d = 40.0 - std::exp((double)rl / (prep->pcr_rate_factor * M_PI)) + 1.0;
        const int rounded = d > 0.0 ? (int)(d + 0.5) : (int)(d - 0.5);
        p.pcr_cache[rl] = (uint8_t)std::max(10, rounded);
    }
    if (prep->dragstr) {
        const ghmm_dragstr &d = *prep->dragstr;
        const size_t cells = (size_t)d.max_period * (size_t)d.max_repeats;
        GHMM_CUDA(b.h_dragstr.reserve(2 * cells), "pinned DRAGstr tables");
        GHMM_CUDA(b.d_dragstr.reserve(2 * cells), "device DRAGstr tables");
        memcpy(b.h_dragstr.p, d.gop, cells * sizeof(double));
        memcpy(b.h_dragstr.p + cells, d.gcp, cells * sizeof(double));
        GHMM_CUDA(cudaMemcpyAsync(b.d_dragstr.p, b.h_dragstr.p, 2 * cells * sizeof(double), cudaMemcpyHostToDevice, s),
                  "H2D DRAGstr tables");
        p.dragstr = 1;
        p.str_gop = b.d_dragstr.p;
        p.str_gcp = b.d_dragstr.p + cells;
        p.str_max_period = d.max_period;
        p.str_max_repeats = d.max_repeats;
        p.max_read_len = max_len;
        b.upload_bytes += (int64_t)(2 * cells * sizeof(double));
    }
    if (!b.prep_events) {
        for (auto &ev : b.ev_prep) GHMM_CUDA(cudaEventCreate(&ev), "cudaEventCreate");
        b.prep_events = true;
    }
    GHMM_CUDA(cudaEventRecord(b.ev_prep[0], s), "event");
    const int e = p.dragstr ? launch_dragstr(b.dev, NR, p, ctx->sm_count, s) : launch_prep(b.dev, NR, p, ctx->sm_count, s);
    if (e) return cuda_fail(ctx, (cudaError_t)e, p.dragstr ? "DRAGstr imputation launch" : "read preparation launch");
    GHMM_CUDA(cudaEventRecord(b.ev_prep[1], s), "event");
    b.prep_timed = true;
    b.upload_bytes += NR * 4;
    return GHMM_OK;
}

void ghmm::set_global_error(const char *msg) {
    std::lock_guard<std::mutex> lk(g_init_error_mu);
    g_init_error = msg ? msg : "";
}

// -------------------------------------------------------------------------------------------------
// C-ABI
extern "C" {

int ghmm_load(void) {
    // test hook: report the hardware as unsupported, as a caller's fallback chain sees it on a machine without one
    const char *unsupported = getenv("GHMM_REPORT_UNSUPPORTED");
    if (unsupported && unsupported[0] && strcmp(unsupported, "0") != 0) return 0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return 0;
    for (int d = 0; d < n; d++) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, d) == cudaSuccess && p.major == 10 && p.minor == 3) return 1;
    }
    return 0;
}

int ghmm_debug_inject(ghmm_ctx *ctx, int32_t kind, int64_t arg) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (arg < 0) return fail(ctx, GHMM_ERR_ARG, "negative injection argument");
    switch (kind) {
        case GHMM_INJECT_REFUSE_ALLOCATIONS: ghmm::g_refuse_allocations.store(arg); return GHMM_OK;
        case GHMM_INJECT_FP64_RERUN_EVERY: ctx->debug_force_rerun = arg; return GHMM_OK;
        default: return fail(ctx, GHMM_ERR_ARG, "unknown injection");
    }
}

int ghmm_initialize(const ghmm_args *args, ghmm_ctx **out) {
    auto set_init_error = [](const std::string &m) {
        std::lock_guard<std::mutex> lk(g_init_error_mu);
        g_init_error = m;
    };
    if (!out) return GHMM_ERR_ARG;
    *out = nullptr;
    ghmm_args a{0, 0, 0, 0};
    if (args) a = *args;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
        set_init_error("no CUDA device available");
        return GHMM_ERR_UNSUPPORTED;
    }
    if (a.device < 0 || a.device >= n) {
        set_init_error("device ordinal out of range");
        return GHMM_ERR_ARG;
    }
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, a.device) != cudaSuccess || !(prop.major == 10 && prop.minor == 3)) {
        set_init_error("device is not compute capability 10.3 (GB300)");
        return GHMM_ERR_UNSUPPORTED;
    }
    auto *ctx = new ghmm_ctx();
    ctx->device = a.device;
    ctx->sm_count = prop.multiProcessorCount;
    ctx->max_threads = a.max_threads;
    ctx->double_precision = a.use_double_precision != 0;
    auto bail = [&](cudaError_t e, const char *what) {
        set_init_error(std::string(what) + ": " + cudaGetErrorString(e));
        delete ctx->host_tables;
        delete ctx;
        return e == cudaErrorMemoryAllocation ? GHMM_ERR_NOMEM : GHMM_ERR_CUDA;
    };
    cudaError_t e = cudaSetDevice(a.device);
    if (e != cudaSuccess) return bail(e, "cudaSetDevice");
    e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) return bail(e, "cudaStreamCreate");
    for (auto &ev : ctx->ev)
        if ((e = cudaEventCreate(&ev)) != cudaSuccess) return bail(e, "cudaEventCreate");
    HostTables *ht = new HostTables();
    build_host_tables(*ht);
    const size_t bytes = sizeof(HostTables);
    e = cudaMalloc(&ctx->table_mem, bytes);
    if (e != cudaSuccess) {
        delete ht;
        return bail(e, "cudaMalloc tables");
    }
    e = cudaMemcpy(ctx->table_mem, ht, bytes, cudaMemcpyHostToDevice);
    ctx->host_tables = ht;
    if (e != cudaSuccess) return bail(e, "upload tables");
    for (int q = 0; q < 256; q++) {
        const double err = ht->err[q], ok = 1.0 - err;
        ctx->expect_log10_prior[q] = (ok > 0.0 ? ok * std::log10(ok) : 0.0) + err * std::log10(err / 3.0);
    }
    const HostTables *dt = (const HostTables *)ctx->table_mem;
    ctx->tables.err_f = dt->err_f;
    ctx->tables.prob_f = dt->prob_f;
    ctx->tables.err3_f = dt->err3_f;
    ctx->tables.m2m_f = dt->m2m_f;
    ctx->tables.err_d = dt->err;
    ctx->tables.prob_d = dt->prob;
    ctx->tables.err3_d = dt->err3;
    ctx->tables.m2m_d = dt->m2m;
    ctx->alive = true;
    *out = ctx;
    return GHMM_OK;
}

// Calibration forward (+ backward): FP32 pass over every pair, then an FP64 pass over the pairs it flagged
// (precision 0), or an FP64 pass over every pair (precision 1).
static int calib_run(ghmm_ctx *ctx, const ghmm_calib_batch *in, int precision, const double *weights, double *loglik,
                     float *gopen, float *gcont, bool backward) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!in || !loglik || (backward && (!gopen || !gcont))) return fail(ctx, GHMM_ERR_ARG, "NULL argument");
    if (precision < 0 || precision > 1) return fail(ctx, GHMM_ERR_ARG, "precision must be 0 (FP32 + FP64 redo) or 1 (FP64)");
    if (in->n_pairs < 0) return fail(ctx, GHMM_ERR_ARG, "negative pair count");
    if (in->n_pairs == 0) return GHMM_OK;
    if (in->max_read_len < 1 || in->max_read_len > 256)
        return fail(ctx, GHMM_ERR_ARG, "calibration supports reads of 1..256 bases (max_read_len)");
    if (in->max_hap_len < 1) return fail(ctx, GHMM_ERR_ARG, "max_hap_len must be >= 1");
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    const int k = (in->max_read_len + 31) / 32;
    const int64_t per_warp = calib_scratch_per_warp(k, in->max_hap_len, true);  // sized for the FP64 pass
    const int64_t warps = (int64_t)calib_grid(ctx->sm_count) * calib_block() / 32;
    if (backward) GHMM_CUDA(ctx->calib_scratch.reserve((size_t)(per_warp * warps)), "calibration scratch");
    GHMM_CUDA(ctx->calib_flags.reserve((size_t)in->n_pairs), "calibration flags");
    cudaStream_t s = ctx->stream;
    if (backward && !weights) {
        GHMM_CUDA(ctx->calib_ones.reserve((size_t)in->n_pairs), "calibration weights");
        std::vector<double> ones((size_t)in->n_pairs, 1.0);
        GHMM_CUDA(cudaMemcpyAsync(ctx->calib_ones.p, ones.data(), ones.size() * 8, cudaMemcpyHostToDevice, s), "H2D weights");
        GHMM_CUDA(cudaStreamSynchronize(s), "H2D weights");
        weights = ctx->calib_ones.p;
    }
    GHMM_CUDA(cudaMemsetAsync(ctx->calib_flags.p, 0, (size_t)in->n_pairs * sizeof(int), s), "clear flags");
    int *flags = ctx->calib_flags.p;
    if (precision == 1) {  // flag every pair so the FP64 pass takes all of them
        std::vector<int> all((size_t)in->n_pairs, 1);
        GHMM_CUDA(cudaMemcpyAsync(flags, all.data(), all.size() * sizeof(int), cudaMemcpyHostToDevice, s), "H2D flags");
        GHMM_CUDA(cudaStreamSynchronize(s), "H2D flags");
    } else {
        int e = launch_calib(ctx->tables, *in, k, backward, false, ctx->calib_scratch.p,
                             calib_scratch_per_warp(k, in->max_hap_len, false), loglik, weights, gopen, gcont, flags,
                             ctx->sm_count, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "calibration FP32 launch");
    }
    int e = launch_calib(ctx->tables, *in, k, backward, true, ctx->calib_scratch.p, per_warp, loglik, weights, gopen,
                         gcont, flags, ctx->sm_count, s);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "calibration FP64 launch");
    GHMM_CUDA(cudaStreamSynchronize(s), "calibration kernels");
    return GHMM_OK;
}

int ghmm_set_tuning(ghmm_ctx *ctx, const ghmm_tuning *t) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!t) return fail(ctx, GHMM_ERR_ARG, "NULL tuning");
    if (ctx->open_queues.load() > (ctx->pipe ? 1 : 0))
        return fail(ctx, GHMM_ERR_STATE, "the tuning cannot change while a queue is open");
    const int mk = t->max_rows_per_lane ? t->max_rows_per_lane : kMaxK32;
    const int mm = t->max_rows_per_lane_multi ? t->max_rows_per_lane_multi : kMaxK32;
    const int cc = t->chunk_cols ? t->chunk_cols : 16384;
    const int rf = t->route_fp64_below ? t->route_fp64_below : kRouteFp64Log10;
    if (mk < 1 || mk > kMaxK32 || mm < 1 || mm > kMaxK32 || cc < 1 || rf > 0)
        return fail(ctx, GHMM_ERR_ARG, "tuning out of range (rows per lane 1..8, chunk_cols >= 1, route_fp64_below <= 0)");
    ctx->max_k = mk;
    ctx->max_k_multi = mm;
    ctx->chunk_cols = cc;
    ctx->route_fp64_log10 = rf;
    return GHMM_OK;
}

int ghmm_done(ghmm_ctx *ctx) {
    if (!ctx) return GHMM_ERR_STATE;
    if (ctx->open_queues.load() > (ctx->pipe ? 1 : 0))
        return fail(ctx, GHMM_ERR_STATE, "destroy the context's queues before ghmm_done");
    cudaSetDevice(ctx->device);
    if (ctx->pipe) queue_close(ctx->pipe);
    ctx->pipe = nullptr;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->scratch_batch.release();
    ctx->pd_batch.release();
    ctx->calib_scratch.release();
    ctx->calib_flags.release();
    ctx->calib_ones.release();
    sw_engine_destroy(ctx->sw);
    ctx->sw = nullptr;
    if (ctx->table_mem) cudaFree(ctx->table_mem);
    delete ctx->host_tables;
    for (auto &ev : ctx->ev)
        if (ev) cudaEventDestroy(ev);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return GHMM_OK;
}

int ghmm_last_error(const ghmm_ctx *ctx, char *buf, size_t n) {
    if (!buf || n == 0) return GHMM_ERR_ARG;
    std::string m;
    if (ctx) {
        m = ctx->last_error;
    } else {
        std::lock_guard<std::mutex> lk(g_init_error_mu);
        m = g_init_error;
    }
    snprintf(buf, n, "%s", m.c_str());
    return GHMM_OK;
}

int ghmm_compute_regions(ghmm_ctx *ctx, const ghmm_region *regions, int32_t n_regions, double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad region array");
    if (n_regions == 0) return GHMM_OK;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    Source src;
    src.regions = regions;
    src.n_regions = n_regions;
    return compute_sync(ctx, src, out);
}

int ghmm_compute_likelihoods(ghmm_ctx *ctx, const ghmm_read *reads, int32_t n_reads, const ghmm_hap *haps,
                             int32_t n_haps, double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (n_reads == 0 || n_haps == 0) return GHMM_OK;  // PairHMM.computeLog10Likelihoods returns early (PairHMM.java:199)
    ghmm_region r{reads, n_reads, haps, n_haps};
    return ghmm_compute_regions(ctx, &r, 1, out);
}

int ghmm_batch_create(ghmm_ctx *ctx, const ghmm_region *regions, int32_t n_regions, ghmm_batch **out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!out || n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    auto *b = new ghmm_batch();
    Source src;
    src.regions = regions;
    src.n_regions = n_regions;
    int rc = batch_marshal(ctx, src, *b);
    if (!rc) rc = batch_upload(ctx, *b, ctx->stream);
    if (!rc) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? GHMM_OK : fail(ctx, GHMM_ERR_CUDA, "upload");
    if (rc) {
        b->release();
        delete b;
        return rc;
    }
    *out = b;
    return GHMM_OK;
}

int ghmm_batch_create_flat(ghmm_ctx *ctx, const ghmm_flat *flat, ghmm_batch **out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!out || !flat || flat->n_regions < 0) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    auto *b = new ghmm_batch();
    Source src;
    src.flat = flat;
    src.n_regions = flat->n_regions;
    int rc = batch_marshal(ctx, src, *b);
    if (!rc) rc = batch_upload(ctx, *b, ctx->stream);
    if (!rc) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? GHMM_OK : fail(ctx, GHMM_ERR_CUDA, "upload");
    if (rc) {
        b->release();
        delete b;
        return rc;
    }
    *out = b;
    return GHMM_OK;
}

int ghmm_batch_forward(ghmm_ctx *ctx, ghmm_batch *b, int32_t mode) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!b) return fail(ctx, GHMM_ERR_ARG, "NULL batch");
    if (mode < 0 || mode > GHMM_MODE_PD_FP32) return fail(ctx, GHMM_ERR_ARG, "unknown mode");
    return batch_forward(ctx, *b, mode);
}

int ghmm_batch_results(ghmm_ctx *ctx, ghmm_batch *b, double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!b) return fail(ctx, GHMM_ERR_ARG, "NULL batch");
    return batch_results(ctx, *b, out);
}

int ghmm_batch_stats(ghmm_ctx *ctx, const ghmm_batch *b, ghmm_stats *st) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!b || !st) return fail(ctx, GHMM_ERR_ARG, "NULL argument");
    st->n_pairs = b->n_out;
    st->n_cells = b->n_cells;
    st->n_rerun = (b->last_mode == GHMM_MODE_FP32_RERUN || b->last_mode == GHMM_MODE_PD_FP32) ? b->last_rerun : 0;
    st->n_fp64_direct = (b->last_mode == GHMM_MODE_FP64 || b->last_mode == GHMM_MODE_PD) ? b->n_out
                        : b->last_mode == GHMM_MODE_PD_FP32                            ? 0
                                                                                       : b->n_direct + b->n_direct_exact;
    st->n_fp64_exact = b->last_mode == GHMM_MODE_PLAIN_FP64 ? 0 : b->last_exact;
    st->n_tasks_fp32 = b->n_tasks;
    st->n_launches = b->last_launches;
    st->reserved = 0;
    st->ms_fp32 = b->ms_fp32;
    st->ms_fp64 = b->ms_fp64;
    st->ms_plain = b->ms_plain;
    st->ms_total = b->ms_total;
    st->h2d_bytes = b->upload_bytes + b->forward_h2d;
    st->d2h_bytes = b->forward_d2h + b->results_d2h;
    st->ms_host_marshal = b->ms_host_copy;
    st->ms_host_tasks = b->ms_host_tasks;
    st->n_cells_fp64_direct = (b->last_mode == GHMM_MODE_FP64 || b->last_mode == GHMM_MODE_PD) ? b->n_cells
                              : (b->last_mode == GHMM_MODE_PD_FP32 || b->last_mode == GHMM_MODE_PLAIN_FP64) ? 0
                                                                                                         : b->cells_direct;
    st->ms_prep = 0.0;
    if (b->prep_timed) {
        float ms = 0.0f;
        GHMM_CUDA(cudaEventSynchronize(b->ev_prep[1]), "event");
        GHMM_CUDA(cudaEventElapsedTime(&ms, b->ev_prep[0], b->ev_prep[1]), "event");
        st->ms_prep = ms;
    }
    return GHMM_OK;
}

int ghmm_batch_postprocess(ghmm_ctx *ctx, ghmm_batch *b, const ghmm_postprocess *pp, uint8_t *keep) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!b || !pp || (b->n_reads > 0 && !keep)) return fail(ctx, GHMM_ERR_ARG, "NULL argument");
    if (!b->uploaded || b->last_mode < 0) return fail(ctx, GHMM_ERR_STATE, "run a forward on the batch first");
    const double cap = pp->max_likelihood_difference_cap;
    if (!(cap < 0.0)) return fail(ctx, GHMM_ERR_ARG, "the minimum reference likelihood fall must be negative");
    if (!(pp->expected_error_rate_per_base >= 0.0)) return fail(ctx, GHMM_ERR_ARG, "expected error rate must be >= 0");
    if (b->n_reads == 0) return GHMM_OK;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    cudaStream_t s = ctx->stream;
    PostArgs p{};
    p.cap = cap;
    p.rate = pp->expected_error_rate_per_base;
    p.scale = pp->read_disqualification_scale;
    p.normalize = std::isinf(cap) ? 0 : 1;
    p.symmetric = pp->symmetric ? 1 : 0;
    p.dynamic = pp->dynamic_disqualification ? 1 : 0;
    if (pp->reference_hap) {
        GHMM_CUDA(b->d_post.reserve((size_t)b->n_regions * sizeof(int32_t) + (size_t)b->n_reads), "device post buffers");
        GHMM_CUDA(cudaMemcpyAsync(b->d_post.p, pp->reference_hap, (size_t)b->n_regions * sizeof(int32_t),
                                  cudaMemcpyHostToDevice, s), "H2D reference haplotypes");
        p.reference_hap = reinterpret_cast<const int32_t *>(b->d_post.p);
    } else {
        GHMM_CUDA(b->d_post.reserve((size_t)b->n_regions * sizeof(int32_t) + (size_t)b->n_reads), "device post buffers");
    }
    uint8_t *d_keep = b->d_post.p + (size_t)b->n_regions * sizeof(int32_t);
    int e = launch_postprocess(b->dev, b->n_reads, p, d_keep, ctx->sm_count, s);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "postprocess launch");
    GHMM_CUDA(cudaMemcpyAsync(keep, d_keep, (size_t)b->n_reads, cudaMemcpyDeviceToHost, s), "D2H keep flags");
    GHMM_CUDA(cudaStreamSynchronize(s), "postprocess");
    return GHMM_OK;
}

int ghmm_batch_destroy(ghmm_ctx *ctx, ghmm_batch *b) {
    if (!b) return GHMM_OK;
    if (ctx) {
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
    }
    b->release();
    delete b;
    return GHMM_OK;
}

int ghmm_compute_flat(ghmm_ctx *ctx, const ghmm_flat *flat, double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!flat || flat->n_regions < 0) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    if (flat->n_regions == 0) return GHMM_OK;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    Source src;
    src.flat = flat;
    src.n_regions = flat->n_regions;
    return compute_sync(ctx, src, out);
}

int ghmm_autotune(ghmm_ctx *ctx, const ghmm_flat *sample, const ghmm_tuning *candidates, int32_t n_candidates,
                  int32_t reps, ghmm_tuning *best, double *ms) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!sample || sample->n_regions <= 0 || n_candidates < 0 || (n_candidates > 0 && !candidates))
        return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    if (ctx->open_queues.load() > (ctx->pipe ? 1 : 0))
        return fail(ctx, GHMM_ERR_STATE, "the tuning cannot change while a queue is open");
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    std::vector<ghmm_tuning> cand;
    if (n_candidates > 0) {
        cand.assign(candidates, candidates + n_candidates);
    } else {  // the built-in grid: rows per lane of single- and multi-strip reads, haplotype columns per task
        for (int mk : {8, 6, 4})
            for (int mm : {8, 6, 4})
                for (int cc : {16384, 4096}) cand.push_back(ghmm_tuning{mk, mm, cc, 0});
    }
    reps = reps > 0 ? reps : 3;
    const int old_k = ctx->max_k, old_m = ctx->max_k_multi, old_c = ctx->chunk_cols;
    const int mode = ctx->double_precision ? GHMM_MODE_FP64 : GHMM_MODE_FP32_RERUN;
    Source src;
    src.flat = sample;
    src.n_regions = sample->n_regions;
    ghmm_batch tb;
    int rc = GHMM_OK, best_i = -1;
    double best_ms = 0;
    for (size_t i = 0; i < cand.size() && !rc; i++) {
        const ghmm_tuning &t = cand[i];
        const int mk = t.max_rows_per_lane ? t.max_rows_per_lane : kMaxK32;
        const int mm = t.max_rows_per_lane_multi ? t.max_rows_per_lane_multi : kMaxK32;
        const int cc = t.chunk_cols ? t.chunk_cols : 16384;
        if (mk < 1 || mk > kMaxK32 || mm < 1 || mm > kMaxK32 || cc < 1) {
            rc = fail(ctx, GHMM_ERR_ARG, "tuning candidate out of range (rows per lane 1..8, chunk_cols >= 1)");
            break;
        }
        ctx->max_k = mk;
        ctx->max_k_multi = mm;
        ctx->chunk_cols = cc;
        rc = batch_marshal(ctx, src, tb);
        if (!rc) rc = batch_upload(ctx, tb, ctx->stream);
        if (!rc) rc = batch_forward(ctx, tb, mode);  // warm-up (graph capture)
        std::vector<double> times;
        for (int r = 0; r < reps && !rc; r++) {
            rc = batch_forward(ctx, tb, mode);
            times.push_back(tb.ms_total);
        }
        if (rc) break;
        std::sort(times.begin(), times.end());
        const double med = times[times.size() / 2];
        if (ms) ms[i] = med;
        if (best_i < 0 || med < best_ms) {
            best_i = (int)i;
            best_ms = med;
        }
        cand[i] = ghmm_tuning{mk, mm, cc, ctx->route_fp64_log10};
    }
    cudaStreamSynchronize(ctx->stream);
    tb.release();
    if (rc || best_i < 0) {
        ctx->max_k = old_k;
        ctx->max_k_multi = old_m;
        ctx->chunk_cols = old_c;
        return rc ? rc : fail(ctx, GHMM_ERR_ARG, "no candidate");
    }
    ctx->max_k = cand[(size_t)best_i].max_rows_per_lane;
    ctx->max_k_multi = cand[(size_t)best_i].max_rows_per_lane_multi;
    ctx->chunk_cols = cand[(size_t)best_i].chunk_cols;
    if (best) *best = cand[(size_t)best_i];
    return GHMM_OK;
}

int ghmm_get_tuning(ghmm_ctx *ctx, ghmm_tuning *t) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!t) return fail(ctx, GHMM_ERR_ARG, "NULL tuning");
    *t = ghmm_tuning{ctx->max_k, ctx->max_k_multi, ctx->chunk_cols, ctx->route_fp64_log10};
    return GHMM_OK;
}

int ghmm_batch_create_raw(ghmm_ctx *ctx, const ghmm_raw_region *regions, int32_t n_regions, const ghmm_read_prep *prep,
                          ghmm_batch **out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!out || n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    RawView v;
    int rc = raw_view(ctx, regions, n_regions, prep, v);
    if (rc) return rc;
    auto *b = new ghmm_batch();
    Source src;
    src.regions = v.regions.data();
    src.n_regions = n_regions;
    src.bound = v.has_bound ? &v.bound : nullptr;
    rc = batch_marshal(ctx, src, *b);
    if (!rc) rc = batch_upload(ctx, *b, ctx->stream);
    if (!rc) rc = raw_prepare_device(ctx, *b, v.mapq.data(), v.max_len, prep, ctx->stream);
    if (!rc) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? GHMM_OK : fail(ctx, GHMM_ERR_CUDA, "upload");
    if (rc) {
        b->release();
        delete b;
        return rc;
    }
    *out = b;
    return GHMM_OK;
}

int ghmm_batch_read_planes(ghmm_ctx *ctx, const ghmm_batch *b, uint8_t *bases, uint8_t *quals, uint8_t *ins,
                           uint8_t *dels, uint8_t *gcp) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!b) return fail(ctx, GHMM_ERR_ARG, "NULL batch");
    if (!b->uploaded) return fail(ctx, GHMM_ERR_STATE, "batch not uploaded");
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    uint8_t *dst[5] = {bases, quals, ins, dels, gcp};
    for (int k = 0; k < 5; k++)
        if (dst[k] && b->read_bytes > 0)
            GHMM_CUDA(cudaMemcpyAsync(dst[k], b->d_planes.p + (size_t)k * b->read_bytes, (size_t)b->read_bytes,
                                      cudaMemcpyDeviceToHost, ctx->stream), "D2H read planes");
    GHMM_CUDA(cudaStreamSynchronize(ctx->stream), "D2H read planes");
    return GHMM_OK;
}

int ghmm_compute_regions_raw(ghmm_ctx *ctx, const ghmm_raw_region *regions, int32_t n_regions, const ghmm_read_prep *prep,
                             double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad region array");
    if (n_regions == 0) return GHMM_OK;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    RawView v;
    int rc = raw_view(ctx, regions, n_regions, prep, v);
    if (rc) return rc;
    Source src;
    src.regions = v.regions.data();
    src.n_regions = n_regions;
    src.bound = v.has_bound ? &v.bound : nullptr;
    {  // large inputs: the pipeline of batches, each prepared on the device after its upload
        std::vector<int64_t> cells, outo;
        if (!region_sizes(src, cells, outo)) return fail(ctx, GHMM_ERR_ARG, "negative count or NULL array in a region");
        int64_t total = 0;
        for (auto c : cells) total += c;
        if (outo.back() > 0 && !out) return fail(ctx, GHMM_ERR_ARG, "NULL output");
        if (total >= kPipelineMinCells && n_regions >= 4)
            return pipelined_compute(ctx, src, cells, outo, out, v.mapq.data(), v.max_len, prep,
                                     v.has_bound ? &v.bound : nullptr);
    }
    ghmm_batch &b = ctx->scratch_batch;
    rc = batch_marshal(ctx, src, b);
    if (!rc) rc = batch_upload(ctx, b, ctx->stream);
    if (!rc) rc = raw_prepare_device(ctx, b, v.mapq.data(), v.max_len, prep, ctx->stream);
    if (!rc) rc = batch_forward(ctx, b, ctx->double_precision ? GHMM_MODE_FP64 : GHMM_MODE_FP32_RERUN);
    if (!rc) rc = batch_results(ctx, b, out);
    return rc;
}

int ghmm_pd_batch_create(ghmm_ctx *ctx, const ghmm_pd_region *regions, int32_t n_regions, ghmm_batch **out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!out || n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto *b = new ghmm_batch();
    int rc = pd_marshal(ctx, regions, n_regions, *b);
    if (!rc) rc = pd_upload(ctx, *b, ctx->stream);
    if (!rc) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? GHMM_OK : fail(ctx, GHMM_ERR_CUDA, "upload");
    if (rc) {
        b->release();
        delete b;
        return rc;
    }
    *out = b;
    return GHMM_OK;
}

int ghmm_pd_compute_regions(ghmm_ctx *ctx, const ghmm_pd_region *regions, int32_t n_regions, double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad region array");
    if (n_regions == 0) return GHMM_OK;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    ghmm_batch &b = ctx->pd_batch;
    int rc = pd_marshal(ctx, regions, n_regions, b);
    if (!rc) rc = pd_upload(ctx, b, ctx->stream);
    if (!rc) rc = batch_forward(ctx, b, ctx->double_precision ? GHMM_MODE_PD : GHMM_MODE_PD_FP32);
    if (!rc) rc = batch_results(ctx, b, out);
    return rc;
}

// PD regions of raw reads: the raw reads' view (checks, 45s and the constant GCP) as the regular raw path builds it,
// then the PD marshal over it, the upload, and the read preparation on the device.
static int pd_raw_build(ghmm_ctx *ctx, const ghmm_pd_raw_region *regions, int32_t n_regions, const ghmm_read_prep *prep,
                        ghmm_batch &b) {
    std::vector<ghmm_raw_region> rr((size_t)n_regions);
    for (int32_t g = 0; g < n_regions; g++) {
        const ghmm_pd_raw_region &rg = regions[g];
        if (rg.n_haps < 0 || (rg.n_haps > 0 && !rg.haps)) return fail(ctx, GHMM_ERR_ARG, "bad PD region");
        rr[(size_t)g] = ghmm_raw_region{rg.reads, rg.n_reads, nullptr, 0};
    }
    RawView v;
    int rc = raw_view(ctx, rr.data(), n_regions, prep, v);
    if (rc) return rc;
    std::vector<ghmm_pd_region> pr((size_t)n_regions);
    for (int32_t g = 0; g < n_regions; g++)
        pr[(size_t)g] = ghmm_pd_region{v.regions[(size_t)g].reads, regions[g].n_reads, regions[g].haps, regions[g].n_haps};
    rc = pd_marshal(ctx, pr.data(), n_regions, b);
    if (!rc) rc = pd_upload(ctx, b, ctx->stream);
    if (!rc) rc = raw_prepare_device(ctx, b, v.mapq.data(), v.max_len, prep, ctx->stream);
    return rc;
}

int ghmm_pd_batch_create_raw(ghmm_ctx *ctx, const ghmm_pd_raw_region *regions, int32_t n_regions,
                             const ghmm_read_prep *prep, ghmm_batch **out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!out || n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto *b = new ghmm_batch();
    int rc = pd_raw_build(ctx, regions, n_regions, prep, *b);
    if (!rc) rc = cudaStreamSynchronize(ctx->stream) == cudaSuccess ? GHMM_OK : fail(ctx, GHMM_ERR_CUDA, "upload");
    if (rc) {
        b->release();
        delete b;
        return rc;
    }
    *out = b;
    return GHMM_OK;
}

int ghmm_pd_compute_regions_raw(ghmm_ctx *ctx, const ghmm_pd_raw_region *regions, int32_t n_regions,
                                const ghmm_read_prep *prep, double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad region array");
    if (n_regions == 0) return GHMM_OK;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    ghmm_batch &b = ctx->pd_batch;
    int rc = pd_raw_build(ctx, regions, n_regions, prep, b);
    if (!rc) rc = batch_forward(ctx, b, ctx->double_precision ? GHMM_MODE_PD : GHMM_MODE_PD_FP32);
    if (!rc) rc = batch_results(ctx, b, out);
    return rc;
}

int ghmm_pd_compute_likelihoods(ghmm_ctx *ctx, const ghmm_read *reads, int32_t n_reads, const ghmm_pd_hap *haps,
                                int32_t n_haps, double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (n_reads == 0 || n_haps == 0) return GHMM_OK;
    ghmm_pd_region r{reads, n_reads, haps, n_haps};
    return ghmm_pd_compute_regions(ctx, &r, 1, out);
}

int ghmm_queue_create(ghmm_ctx *ctx, int64_t batch_cells, ghmm_queue **queue) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!queue || batch_cells < 0) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    *queue = nullptr;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    return queue_open(ctx, batch_cells, queue);
}

int ghmm_queue_create_raw(ghmm_ctx *ctx, int64_t batch_cells, const ghmm_read_prep *prep, ghmm_queue **queue) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!queue || batch_cells < 0) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    *queue = nullptr;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    RawView v;  // checks the preparation arguments (no regions)
    const int rc = raw_view(ctx, nullptr, 0, prep, v);
    if (rc) return rc;
    return queue_open(ctx, batch_cells, queue, prep, v.has_bound ? &v.bound : nullptr);
}

int ghmm_queue_push_raw(ghmm_queue *q, const ghmm_raw_region *regions, int32_t n_regions, double *out) {
    if (!q) return GHMM_ERR_STATE;
    ghmm_ctx *ctx = q->ctx;
    if (int rc = queue_status(q)) return rc;
    if (!q->raw) return fail(ctx, GHMM_ERR_STATE, "raw reads go to a queue made by ghmm_queue_create_raw");
    if (n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad region array");
    // check everything first, so that a rejected push leaves the queue as it was
    int64_t n_out = 0;
    for (int32_t g = 0; g < n_regions; g++) {
        const ghmm_raw_region &rg = regions[g];
        int32_t max_len = 0;
        if (const int e = raw_region_problem(rg, &max_len)) return fail(ctx, GHMM_ERR_ARG, kRawErrors[e]);
        if (q->prep.dragstr && max_len > kDragstrMaxRead)
            return fail(ctx, GHMM_ERR_ARG, "the DRAGstr imputation takes reads of up to 28000 bases");
        for (int32_t r = 0; r < rg.n_reads; r++) {
            const ghmm_raw_read &rd = rg.reads[r];
            for (int32_t i = 0; i < rd.length; i++)
                if (rd.quals[i] > kMaxQual || (rd.ins_quals && rd.ins_quals[i] > 127) ||
                    (rd.del_quals && rd.del_quals[i] > 127))
                    return fail(ctx, GHMM_ERR_ARG,
                                "quality out of range (base quality must be <= 254; insertion and deletion qualities "
                                "0..127)");
        }
        for (int32_t h = 0; h < rg.n_haps; h++) {
            const ghmm_hap &hp = rg.haps[h];
            if (hp.length < 0 || hp.length > kMaxHapLen) return fail(ctx, GHMM_ERR_ARG, "haplotype length out of range");
            if (hp.length > 0 && !hp.bases) return fail(ctx, GHMM_ERR_ARG, "NULL haplotype bases");
        }
        n_out += (int64_t)rg.n_reads * rg.n_haps;
    }
    if (n_out > 0 && !out) return fail(ctx, GHMM_ERR_ARG, "NULL output");
    if (!q->open) q->open = std::make_unique<QueueUnit>();
    QueueUnit &u = *q->open;
    for (int32_t g = 0; g < n_regions; g++) {
        const ghmm_raw_region &rg = regions[g];
        int64_t sr = 0, sh = 0;
        for (int32_t r = 0; r < rg.n_reads; r++) {
            const ghmm_raw_read &rd = rg.reads[r];
            const size_t L = (size_t)rd.length;
            u.planes[0].insert(u.planes[0].end(), rd.bases, rd.bases + L);
            u.planes[1].insert(u.planes[1].end(), rd.quals, rd.quals + L);
            if (rd.ins_quals) u.planes[2].insert(u.planes[2].end(), rd.ins_quals, rd.ins_quals + L);
            else u.planes[2].resize(u.planes[2].size() + L, 45);  // ReadUtils.DEFAULT_INSERTION_DELETION_QUAL
            if (rd.del_quals) u.planes[3].insert(u.planes[3].end(), rd.del_quals, rd.del_quals + L);
            else u.planes[3].resize(u.planes[3].size() + L, 45);
            u.planes[4].resize(u.planes[4].size() + L, (uint8_t)q->prep.gcp);
            u.read_off.push_back(u.read_off.back() + rd.length);
            u.mapq.push_back(rd.mapping_quality);
            u.max_len = std::max(u.max_len, rd.length);
            sr += rd.length;
        }
        for (int32_t h = 0; h < rg.n_haps; h++) {
            const ghmm_hap &hp = rg.haps[h];
            u.hap_bases.insert(u.hap_bases.end(), hp.bases, hp.bases + hp.length);
            u.hap_off.push_back(u.hap_off.back() + hp.length);
            sh += hp.length;
        }
        u.region_read_off.push_back(u.region_read_off.back() + rg.n_reads);
        u.region_hap_off.push_back(u.region_hap_off.back() + rg.n_haps);
        u.n_regions++;
        u.cells += sr * sh;
        std::lock_guard<std::mutex> lk(q->mu);
        q->info.n_cells += sr * sh;
    }
    if (n_out > 0) {
        if (!u.dests.empty() && u.dests.back().first + u.dests.back().second == out)
            u.dests.back().second += n_out;  // contiguous with the previous push
        else
            u.dests.emplace_back(out, n_out);
    }
    u.n_out += n_out;
    {
        std::lock_guard<std::mutex> lk(q->mu);
        q->info.n_regions += n_regions;
        q->info.n_pairs += n_out;
    }
    if (u.cells >= q->batch_cells) queue_submit(q, std::move(q->open));
    return queue_status(q);
}

int ghmm_queue_push(ghmm_queue *q, const ghmm_region *regions, int32_t n_regions, double *out) {
    if (!q) return GHMM_ERR_STATE;
    ghmm_ctx *ctx = q->ctx;
    if (int rc = queue_status(q)) return rc;
    if (q->raw) return fail(ctx, GHMM_ERR_STATE, "a raw queue takes ghmm_queue_push_raw");
    if (n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad region array");
    // check everything first, so that a rejected push leaves the queue as it was
    int64_t n_out = 0;
    for (int32_t g = 0; g < n_regions; g++) {
        const ghmm_region &rg = regions[g];
        if (rg.n_reads < 0 || rg.n_haps < 0) return fail(ctx, GHMM_ERR_ARG, "negative read or haplotype count");
        if ((rg.n_reads > 0 && !rg.reads) || (rg.n_haps > 0 && !rg.haps))
            return fail(ctx, GHMM_ERR_ARG, "NULL read or haplotype array");
        for (int32_t r = 0; r < rg.n_reads; r++) {
            const ghmm_read &rd = rg.reads[r];
            if (rd.length < 0 || rd.length > kMaxReadLen) return fail(ctx, GHMM_ERR_ARG, "read length out of range");
            if (rd.length > 0 && (!rd.bases || !rd.quals || !rd.ins_gop || !rd.del_gop || !rd.gcp))
                return fail(ctx, GHMM_ERR_ARG, "NULL read array");
            for (int32_t i = 0; i < rd.length; i++)
                if (rd.quals[i] > kMaxQual || rd.ins_gop[i] > 127 || rd.del_gop[i] > 127 || rd.gcp[i] > 127)
                    return fail(ctx, GHMM_ERR_ARG,
                                "quality out of range (base quality must be <= 254; insertion, deletion and gap "
                                "continuation penalties must be 0..127)");
        }
        for (int32_t h = 0; h < rg.n_haps; h++) {
            const ghmm_hap &hp = rg.haps[h];
            if (hp.length < 0 || hp.length > kMaxHapLen) return fail(ctx, GHMM_ERR_ARG, "haplotype length out of range");
            if (hp.length > 0 && !hp.bases) return fail(ctx, GHMM_ERR_ARG, "NULL haplotype bases");
        }
        n_out += (int64_t)rg.n_reads * rg.n_haps;
    }
    if (n_out > 0 && !out) return fail(ctx, GHMM_ERR_ARG, "NULL output");
    if (!q->open) q->open = std::make_unique<QueueUnit>();
    QueueUnit &u = *q->open;
    for (int32_t g = 0; g < n_regions; g++) {
        const ghmm_region &rg = regions[g];
        int64_t sr = 0, sh = 0;
        for (int32_t r = 0; r < rg.n_reads; r++) {
            const ghmm_read &rd = rg.reads[r];
            const uint8_t *src[5] = {rd.bases, rd.quals, rd.ins_gop, rd.del_gop, rd.gcp};
            for (int p = 0; p < 5; p++) u.planes[p].insert(u.planes[p].end(), src[p], src[p] + rd.length);
            u.read_off.push_back(u.read_off.back() + rd.length);
            sr += rd.length;
        }
        for (int32_t h = 0; h < rg.n_haps; h++) {
            const ghmm_hap &hp = rg.haps[h];
            u.hap_bases.insert(u.hap_bases.end(), hp.bases, hp.bases + hp.length);
            u.hap_off.push_back(u.hap_off.back() + hp.length);
            sh += hp.length;
        }
        u.region_read_off.push_back(u.region_read_off.back() + rg.n_reads);
        u.region_hap_off.push_back(u.region_hap_off.back() + rg.n_haps);
        u.n_regions++;
        u.cells += sr * sh;
        std::lock_guard<std::mutex> lk(q->mu);
        q->info.n_cells += sr * sh;
    }
    if (n_out > 0) {
        if (!u.dests.empty() && u.dests.back().first + u.dests.back().second == out)
            u.dests.back().second += n_out;  // contiguous with the previous push
        else
            u.dests.emplace_back(out, n_out);
    }
    u.n_out += n_out;
    {
        std::lock_guard<std::mutex> lk(q->mu);
        q->info.n_regions += n_regions;
        q->info.n_pairs += n_out;
    }
    if (u.cells >= q->batch_cells) queue_submit(q, std::move(q->open));
    return queue_status(q);
}

int ghmm_queue_flush(ghmm_queue *q) {
    if (!q) return GHMM_ERR_STATE;
    if (q->open && q->open->n_regions > 0) queue_submit(q, std::move(q->open));
    q->open.reset();
    queue_wait_all(q);
    return queue_status(q);
}

int ghmm_queue_get_info(ghmm_queue *q, ghmm_queue_info *info) {
    if (!q) return GHMM_ERR_STATE;
    if (!info) return fail(q->ctx, GHMM_ERR_ARG, "NULL info");
    std::lock_guard<std::mutex> lk(q->mu);
    *info = q->info;
    return GHMM_OK;
}

int ghmm_queue_destroy(ghmm_queue *q) {
    if (!q) return GHMM_OK;
    if (q->open && q->open->n_regions > 0) queue_submit(q, std::move(q->open));
    queue_wait_all(q);
    queue_close(q);
    return GHMM_OK;
}

void *ghmm_stream(ghmm_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int ghmm_calib_forward(ghmm_ctx *ctx, const ghmm_calib_batch *batch, int32_t precision, double *d_loglik) {
    return calib_run(ctx, batch, precision, nullptr, d_loglik, nullptr, nullptr, false);
}

int ghmm_calib_backward(ghmm_ctx *ctx, const ghmm_calib_batch *batch, int32_t precision, const double *d_weights,
                        double *d_loglik, float *d_grad_open, float *d_grad_cont) {
    return calib_run(ctx, batch, precision, d_weights, d_loglik, d_grad_open, d_grad_cont, true);
}

int ghmm_measure_peaks(ghmm_ctx *ctx, double *fp32, double *fp32x2, double *fp64) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    double a = 0, b = 0, c = 0;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    int e = measure_peaks_device(ctx->sm_count, &a, &b, &c, ctx->stream);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "peak probes");
    if (fp32) *fp32 = a;
    if (fp32x2) *fp32x2 = b;
    if (fp64) *fp64 = c;
    return GHMM_OK;
}

int ghmm_debug_tables(ghmm_ctx *ctx, double *err, double *prob, double *m2m) {
    if (!ctx) {  // host-built tables, no device needed
        HostTables *ht = new HostTables();
        build_host_tables(*ht);
        if (err) memcpy(err, ht->err, sizeof ht->err);
        if (prob) memcpy(prob, ht->prob, sizeof ht->prob);
        if (m2m) memcpy(m2m, ht->m2m, sizeof ht->m2m);
        delete ht;
        return GHMM_OK;
    }
    if (!ctx->alive) return GHMM_ERR_STATE;
    const HostTables *dt = (const HostTables *)ctx->table_mem;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    if (err) GHMM_CUDA(cudaMemcpy(err, dt->err, 256 * sizeof(double), cudaMemcpyDeviceToHost), "D2H tables");
    if (prob) GHMM_CUDA(cudaMemcpy(prob, dt->prob, 256 * sizeof(double), cudaMemcpyDeviceToHost), "D2H tables");
    if (m2m) GHMM_CUDA(cudaMemcpy(m2m, dt->m2m, 128 * 128 * sizeof(double), cudaMemcpyDeviceToHost), "D2H tables");
    return GHMM_OK;
}

}  // extern "C"

namespace ghmm {

int ctx_info(ghmm_ctx *ctx, CtxInfo *info) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    info->device = ctx->device;
    info->sm_count = ctx->sm_count;
    info->threads = hw_threads(ctx->max_threads);
    info->stream = ctx->stream;
    info->sw = &ctx->sw;
    return GHMM_OK;
}

int ctx_fail(ghmm_ctx *ctx, int code, const std::string &msg) { return fail(ctx, code, msg); }

void batch_info(const ghmm_batch *b, BatchInfo *info) {
    info->dev = &b->dev;
    info->h_off = b->h_off.p;
    info->n_regions = b->n_regions;
    info->n_reads = b->n_reads;
    info->n_haps = b->n_haps;
    info->has_results = b->uploaded && b->last_mode >= 0;
}

}  // namespace ghmm
