// runtime.cpp -- host runtime and C-ABI of the GB300 PairHMM (include/ghmm.h).
//
// A call flows: marshal (multi-threaded copy of every read's five byte arrays and every haplotype into
// pinned planes, haplotype column codes, validation) -> build warp tasks (reads paired within a region
// by rows-per-lane bucket, longest first) -> async H2D -> FP32 bucket launches -> FP64 queue launch ->
// D2H -> validation of results (log10 L <= 0, not NaN; PairHMM.java:305-306).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ghmm.h"
#include "ghmm_internal.h"
#include "tables.h"

using namespace ghmm;

namespace {

std::mutex g_init_error_mu;
std::string g_init_error;

constexpr int kBlock = 128;
constexpr int kWarpsPerBlock = kBlock / 32;
constexpr int kCounterBase = 8;  // counters[8 + bucket] are per-bucket task cursors
constexpr int kNumCounters = 64;

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

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(n, 1);
        cudaError_t e = cudaMalloc(&p, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
    }
};

template <typename T>
struct HostBuf {  // pinned
    T *p = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        const size_t want = std::max<size_t>(n, 1);
        cudaError_t e = cudaMallocHost(&p, want * sizeof(T));
        if (e == cudaSuccess) cap = want;
        return e;
    }
    void release() {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

int hw_threads(int requested) {
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    return requested > 0 ? std::min(requested, hw) : hw;
}

template <typename F>
void parallel_for(int64_t n, int threads, F f) {
    if (n <= 0) return;
    threads = (int)std::min<int64_t>(threads, n);
    if (threads <= 1) {
        for (int64_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<int64_t> next{0};
    std::vector<std::thread> pool;
    for (int t = 0; t < threads; t++)
        pool.emplace_back([&] {
            for (;;) {
                const int64_t i0 = next.fetch_add(64);
                if (i0 >= n) break;
                const int64_t i1 = std::min(n, i0 + 64);
                for (int64_t i = i0; i < i1; i++) f(i);
            }
        });
    for (auto &th : pool) th.join();
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
    HostBuf<uint8_t> h_hap;     // raw bytes then codes
    HostBuf<int64_t> h_off;     // read_off | hap_off | region_read_off | region_hap_off | out_off
    HostBuf<int32_t> h_read_region;
    HostBuf<float> h_init_f;
    HostBuf<double> h_init_d;
    HostBuf<F32Task> h_tasks;
    HostBuf<PairRef> h_direct;
    HostBuf<double> h_out;
    HostBuf<int32_t> h_counters;
    // device
    DevBuf<uint8_t> d_planes, d_hap;
    DevBuf<int64_t> d_off;
    DevBuf<int32_t> d_read_region;
    DevBuf<float> d_init_f;
    DevBuf<double> d_init_d;
    DevBuf<F32Task> d_tasks;
    DevBuf<PairRef> d_rerun;
    DevBuf<double> d_out;
    DevBuf<int32_t> d_counters;
    DevBuf<float2> d_scratch32;
    DevBuf<double> d_scratch64;
    // sizes
    int64_t n_regions = 0, n_reads = 0, n_haps = 0, read_bytes = 0, hap_bytes = 0, n_out = 0;
    int64_t n_cells = 0;
    int max_read_len = 0, max_hap_len = 0;
    std::vector<int> region_max_read;  // for the plain kernel's shared-memory size
    // tasks
    std::vector<Bucket> buckets;
    int64_t n_tasks = 0, n_direct = 0;
    int64_t n_direct_fp64mode = 0;
    int64_t scratch32_cols = 0;
    int fp64_grid = 0;
    // last forward
    int last_mode = -1;
    int last_launches = 0;
    int64_t last_rerun = 0;
    double ms_fp32 = 0, ms_fp64 = 0, ms_plain = 0, ms_total = 0;
    int64_t upload_bytes = 0, forward_h2d = 0, forward_d2h = 0, results_d2h = 0;
    bool uploaded = false;
    DevBatch dev{};

    void release() {
        h_planes.release(); h_hap.release(); h_off.release(); h_read_region.release(); h_init_f.release();
        h_init_d.release(); h_tasks.release(); h_direct.release(); h_out.release(); h_counters.release();
        d_planes.release(); d_hap.release(); d_off.release(); d_read_region.release(); d_init_f.release();
        d_init_d.release(); d_tasks.release(); d_rerun.release(); d_out.release(); d_counters.release();
        d_scratch32.release(); d_scratch64.release();
    }
};

struct ghmm_ctx {
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
    int max_k = kMaxK32, max_k_multi = kMaxK32, chunk_cols = 16384;
    // calibration scratch (checkpointed fronts per resident warp), FP64-redo flags, unit weights
    DevBuf<uint8_t> calib_scratch;
    DevBuf<int> calib_flags;
    DevBuf<double> calib_ones;
    bool alive = false;
};

namespace {

int fail(ghmm_ctx *ctx, int code, const std::string &msg) {
    if (ctx) ctx->last_error = msg;
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
struct Source {
    // either regions (per-read pointers) ...
    const ghmm_region *regions = nullptr;
    int64_t n_regions = 0;
    // ... or flat planes
    const ghmm_flat *flat = nullptr;
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
    std::vector<int64_t> read_off, hap_off, rro, rho, oo;
    int rc = plan_sizes(ctx, src, b, read_off, hap_off, rro, rho, oo);
    if (rc) return rc;
    const int64_t G = b.n_regions, NR = b.n_reads, NH = b.n_haps;
    const int threads = hw_threads(ctx->max_threads);

    GHMM_CUDA(b.h_planes.reserve((size_t)b.read_bytes * 5), "pinned read planes");
    GHMM_CUDA(b.h_hap.reserve((size_t)b.hap_bytes * 2), "pinned haplotypes");
    const size_t n_off = (size_t)(NR + 1) + (size_t)(NH + 1) + 3 * (size_t)(G + 1);
    GHMM_CUDA(b.h_off.reserve(n_off), "pinned offsets");
    GHMM_CUDA(b.h_read_region.reserve((size_t)NR), "pinned read regions");
    GHMM_CUDA(b.h_init_f.reserve((size_t)NH), "pinned init");
    GHMM_CUDA(b.h_init_d.reserve((size_t)NH), "pinned init");
    GHMM_CUDA(b.h_counters.reserve(kNumCounters), "pinned counters");

    uint8_t *P = b.h_planes.p;
    const int64_t RB = b.read_bytes;
    uint8_t *pb = P, *pq = P + RB, *pi = P + 2 * RB, *pd = P + 3 * RB, *pg = P + 4 * RB;
    uint8_t *hraw = b.h_hap.p, *hcode = b.h_hap.p + b.hap_bytes;
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
            double growth = 1.0;
            for (int i = 0; i < R; i++) {
                if (sq[i] > kMaxQual || si[i] > 127 || sd[i] > 127 || sg[i] > 127) {
                    fl |= 2;
                    break;
                }
                if (sg[i] == 0 || base_code(sb[i]) == 0) fl |= 1;
                const double mm = HT.m2m[si[i] * 128 + sd[i]];
                if (mm < 1e-6) fl |= 1;
                if (i > 0) {
                    const double e = HT.err[sg[i]] * HT.err[si[i - 1]] /
                                     (HT.err[si[i]] * std::max(HT.m2m[si[i - 1] * 128 + sd[i - 1]], 1e-300));
                    growth = 1.0 + e * growth;
                    if (growth > max_i_scaled) fl |= 1;
                }
            }
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
    // ceil(R/256) strips, paired within a region and bucket, and split into haplotype chunks.
    std::vector<std::vector<F32Task>> per_bucket(32);
    std::vector<std::vector<int64_t>> per_bucket_cost(32);
    std::vector<PairRef> direct;
    int64_t max_multi_cols = 0;
    for (int64_t g = 0; g < G; g++) {
        const int64_t h0 = rho[(size_t)g], h1 = rho[(size_t)g + 1];
        const int64_t r0 = rro[(size_t)g], r1 = rro[(size_t)g + 1];
        if (h1 == h0 || r1 == r0) continue;
        bool region_fp64 = false;
        for (int64_t h = h0; h < h1; h++) region_fp64 |= (hap_flag[(size_t)h] != 0);
        std::vector<std::pair<int64_t, int64_t>> groups;  // ((key, strips, length), read)
        for (int64_t r = r0; r < r1; r++) {
            const int R = (int)(read_off[(size_t)r + 1] - read_off[(size_t)r]);
            if (region_fp64 || (read_flag[(size_t)r] & 1)) {
                for (int64_t h = h0; h < h1; h++) direct.push_back(PairRef{(int32_t)r, (int32_t)h});
                continue;
            }
            int key, ns = 1;
            if (R <= 32 * ctx->max_k) {
                key = (R + 31) / 32;
            } else {  // fewest strips of at most max_k_multi rows per lane, then the fewest rows per lane
                ns = (R + 32 * ctx->max_k_multi - 1) / (32 * ctx->max_k_multi);
                key = ((R + 32 * ns - 1) / (32 * ns)) | 16;
            }
            // reads are paired only within one (rows per lane, strip count) class
            groups.emplace_back(((int64_t)key * 4096 + ns) * 100000 + R, r);
        }
        std::sort(groups.begin(), groups.end());
        // haplotype chunks
        std::vector<std::pair<int64_t, int64_t>> chunks;
        {
            int64_t a = h0;
            while (a < h1) {
                int64_t e = a + 1, cols = hap_off[(size_t)a + 1] - hap_off[(size_t)a];
                while (e < h1 && cols + (hap_off[(size_t)e + 1] - hap_off[(size_t)e]) <= ctx->chunk_cols) {
                    cols += hap_off[(size_t)e + 1] - hap_off[(size_t)e];
                    e++;
                }
                chunks.emplace_back(a, e);
                a = e;
            }
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
            const int nstrips = multi ? (std::max(Ra, Rb) + S - 1) / S : 1;
            for (auto &ch : chunks) {
                F32Task t;
                t.read_a = (int32_t)ra;
                t.read_b = (int32_t)rb;
                t.hap_begin = (int32_t)ch.first;
                t.hap_end = (int32_t)ch.second;
                t.region = (int32_t)g;
                t.nstrips = (int16_t)nstrips;
                t.k = (int16_t)K;
                t.pad_a = nstrips * S - Ra;
                t.pad_b = rb >= 0 ? nstrips * S - Rb : nstrips * S;
                const int64_t cols = hap_off[(size_t)ch.second] - hap_off[(size_t)ch.first];
                if (multi) max_multi_cols = std::max(max_multi_cols, cols);
                per_bucket[(size_t)key].push_back(t);
                per_bucket_cost[(size_t)key].push_back((cols + 31) * K * nstrips);
            }
        }
    }
    // order each bucket longest first and concatenate
    b.buckets.clear();
    int64_t total_tasks = 0;
    for (auto &v : per_bucket) total_tasks += (int64_t)v.size();
    GHMM_CUDA(b.h_tasks.reserve((size_t)total_tasks), "pinned tasks");
    int64_t pos = 0;
    for (int key = 1; key < 32; key++) {
        auto &v = per_bucket[(size_t)key];
        if (v.empty()) continue;
        auto &cost = per_bucket_cost[(size_t)key];
        std::vector<size_t> idx(v.size());
        std::iota(idx.begin(), idx.end(), 0);
        std::stable_sort(idx.begin(), idx.end(), [&](size_t x, size_t y) { return cost[x] > cost[y]; });
        for (size_t k = 0; k < idx.size(); k++) b.h_tasks.p[pos + (int64_t)k] = v[idx[k]];
        int bpsm = 0;
        if (fp32_kernel_occupancy(key, kBlock, &bpsm) != 0 || bpsm <= 0) bpsm = 1;
        const int64_t want = ((int64_t)v.size() + kWarpsPerBlock - 1) / kWarpsPerBlock;
        const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->sm_count * bpsm));
        b.buckets.push_back(Bucket{key, (int)pos, (int)v.size(), grid});
        pos += (int64_t)v.size();
    }
    b.n_tasks = total_tasks;
    b.n_direct = (int64_t)direct.size();
    GHMM_CUDA(b.h_direct.reserve(direct.size()), "pinned direct pairs");
    if (!direct.empty()) memcpy(b.h_direct.p, direct.data(), direct.size() * sizeof(PairRef));
    b.scratch32_cols = max_multi_cols;
    int bpsm64 = 0;
    if (fp64_kernel_occupancy(kBlock, &bpsm64) != 0 || bpsm64 <= 0) bpsm64 = 1;
    b.fp64_grid = ctx->sm_count * bpsm64;
    b.uploaded = false;
    return GHMM_OK;
}

// Allocate device buffers and upload the staged batch.
static int batch_upload(ghmm_ctx *ctx, ghmm_batch &b) {
    const int64_t NR = b.n_reads, NH = b.n_haps, G = b.n_regions;
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    GHMM_CUDA(b.d_planes.reserve((size_t)b.read_bytes * 5), "device read planes");
    GHMM_CUDA(b.d_hap.reserve((size_t)b.hap_bytes * 2), "device haplotypes");
    const size_t n_off = (size_t)(NR + 1) + (size_t)(NH + 1) + 3 * (size_t)(G + 1);
    GHMM_CUDA(b.d_off.reserve(n_off), "device offsets");
    GHMM_CUDA(b.d_read_region.reserve((size_t)NR), "device read regions");
    GHMM_CUDA(b.d_init_f.reserve((size_t)NH), "device init");
    GHMM_CUDA(b.d_init_d.reserve((size_t)NH), "device init");
    GHMM_CUDA(b.d_tasks.reserve((size_t)b.n_tasks), "device tasks");
    const int64_t capacity = std::max<int64_t>(b.n_out, 1);
    GHMM_CUDA(b.d_rerun.reserve((size_t)capacity), "device FP64 queue");
    GHMM_CUDA(b.d_out.reserve((size_t)std::max<int64_t>(b.n_out, 1)), "device output");
    GHMM_CUDA(b.d_counters.reserve(kNumCounters), "device counters");
    int max_grid_multi = 0;
    for (auto &bk : b.buckets)
        if (bk.key & 16) max_grid_multi = std::max(max_grid_multi, bk.grid);
    const size_t s32 = (size_t)max_grid_multi * kWarpsPerBlock * (size_t)b.scratch32_cols * 3;
    GHMM_CUDA(b.d_scratch32.reserve(std::max<size_t>(s32, 1)), "device FP32 strip scratch");
    const size_t s64 = (size_t)b.fp64_grid * kWarpsPerBlock * (size_t)std::max(b.max_hap_len, 1) * 3;
    GHMM_CUDA(b.d_scratch64.reserve(s64), "device FP64 strip scratch");

    cudaStream_t s = ctx->stream;
    GHMM_CUDA(cudaMemcpyAsync(b.d_planes.p, b.h_planes.p, (size_t)b.read_bytes * 5, cudaMemcpyHostToDevice, s), "H2D planes");
    GHMM_CUDA(cudaMemcpyAsync(b.d_hap.p, b.h_hap.p, (size_t)b.hap_bytes * 2, cudaMemcpyHostToDevice, s), "H2D haplotypes");
    GHMM_CUDA(cudaMemcpyAsync(b.d_off.p, b.h_off.p, n_off * sizeof(int64_t), cudaMemcpyHostToDevice, s), "H2D offsets");
    if (NR) GHMM_CUDA(cudaMemcpyAsync(b.d_read_region.p, b.h_read_region.p, (size_t)NR * 4, cudaMemcpyHostToDevice, s), "H2D regions");
    if (NH) {
        GHMM_CUDA(cudaMemcpyAsync(b.d_init_f.p, b.h_init_f.p, (size_t)NH * 4, cudaMemcpyHostToDevice, s), "H2D init");
        GHMM_CUDA(cudaMemcpyAsync(b.d_init_d.p, b.h_init_d.p, (size_t)NH * 8, cudaMemcpyHostToDevice, s), "H2D init");
    }
    if (b.n_tasks)
        GHMM_CUDA(cudaMemcpyAsync(b.d_tasks.p, b.h_tasks.p, (size_t)b.n_tasks * sizeof(F32Task), cudaMemcpyHostToDevice, s), "H2D tasks");

    b.upload_bytes = b.read_bytes * 5 + b.hap_bytes * 2 + (int64_t)n_off * 8 + NR * 4 + NH * 12 +
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
    d.hap_code = b.d_hap.p + b.hap_bytes;
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
    d.rerun_capacity = capacity;
    d.scratch32 = b.d_scratch32.p;
    d.scratch32_cols = b.scratch32_cols;
    d.scratch64 = b.d_scratch64.p;
    d.scratch64_cols = std::max(b.max_hap_len, 1);
    b.uploaded = true;
    return GHMM_OK;
}

// Direct FP64 pairs: all pairs (FP64 mode) or the host-classified ones.
static int fill_fp64_all(ghmm_ctx *ctx, ghmm_batch &b) {
    // every (read, hap) pair of every region, read-major
    GHMM_CUDA(b.h_direct.reserve((size_t)std::max<int64_t>(b.n_out, 1)), "pinned FP64 pairs");
    const int64_t *o = b.h_off.p;
    const int64_t NR = b.n_reads, NH = b.n_haps, G = b.n_regions;
    const int64_t *rro = o + NR + 1 + NH + 1, *rho = rro + G + 1;
    int64_t k = 0;
    for (int64_t g = 0; g < G; g++)
        for (int64_t r = rro[g]; r < rro[g + 1]; r++)
            for (int64_t h = rho[g]; h < rho[g + 1]; h++) b.h_direct.p[k++] = PairRef{(int32_t)r, (int32_t)h};
    b.n_direct_fp64mode = k;
    return GHMM_OK;
}

static int batch_forward(ghmm_ctx *ctx, ghmm_batch &b, int mode) {
    if (!b.uploaded) return fail(ctx, GHMM_ERR_STATE, "batch not uploaded");
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
            return fail(ctx, GHMM_ERR_ARG, "the plain FP64 kernel supports reads up to 1024 bases");
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
    // counters: cursors 0, FP64 queue tail = number of pre-queued pairs
    int64_t n_pre = b.n_direct;
    if (mode == GHMM_MODE_FP64) {
        if (b.n_direct_fp64mode != b.n_out) {
            int rc = fill_fp64_all(ctx, b);
            if (rc) return rc;
        }
        n_pre = b.n_direct_fp64mode;
    }
    if (n_pre > 0)
        GHMM_CUDA(cudaMemcpyAsync(b.d_rerun.p, b.h_direct.p, (size_t)n_pre * sizeof(PairRef), cudaMemcpyHostToDevice, s),
                  "H2D FP64 pairs");
    b.forward_h2d = n_pre * (int64_t)sizeof(PairRef) + kNumCounters * 4;
    b.forward_d2h = kNumCounters * 4;
    int32_t *hc = b.h_counters.p;
    for (int i = 0; i < kNumCounters; i++) hc[i] = 0;
    hc[1] = (int32_t)n_pre;
    GHMM_CUDA(cudaMemcpyAsync(b.d_counters.p, hc, kNumCounters * sizeof(int32_t), cudaMemcpyHostToDevice, s), "H2D counters");
    GHMM_CUDA(cudaEventRecord(ev[2], s), "event");
    if (mode == GHMM_MODE_FP32_RERUN) {
        int slot = kCounterBase;
        for (auto &bk : b.buckets) {
            int e = launch_fp32_bucket(ctx->tables, b.dev, bk.key, bk.begin, bk.count, bk.grid, kBlock, slot++, s);
            if (e) return cuda_fail(ctx, (cudaError_t)e, "FP32 bucket launch");
            b.last_launches++;
        }
    }
    if (mode == GHMM_MODE_FP32_RERUN && b.n_tasks > 0) {
        int e = launch_finalize_fp32(b.dev.out, b.n_out, ctx->sm_count, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "FP32 finalize launch");
        b.last_launches++;
    }
    GHMM_CUDA(cudaEventRecord(ev[3], s), "event");
    {
        int e = launch_fp64_queue(ctx->tables, b.dev, b.fp64_grid, kBlock, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "FP64 queue launch");
        b.last_launches++;
    }
    GHMM_CUDA(cudaEventRecord(ev[4], s), "event");
    GHMM_CUDA(cudaMemcpyAsync(hc, b.d_counters.p, kNumCounters * sizeof(int32_t), cudaMemcpyDeviceToHost, s), "D2H counters");
    GHMM_CUDA(cudaStreamSynchronize(s), "forward kernels");
    float ms = 0;
    cudaEventElapsedTime(&ms, ev[2], ev[3]);
    b.ms_fp32 = ms;
    cudaEventElapsedTime(&ms, ev[3], ev[4]);
    b.ms_fp64 = ms;
    cudaEventElapsedTime(&ms, ev[0], ev[4]);
    b.ms_total = ms;
    if (hc[3] != 0) return fail(ctx, GHMM_ERR_CUDA, "device-side queue overflow or scratch bound exceeded");
    b.last_rerun = (int64_t)hc[1] - n_pre;
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

void ghmm::set_global_error(const char *msg) {
    std::lock_guard<std::mutex> lk(g_init_error_mu);
    g_init_error = msg ? msg : "";
}

// -------------------------------------------------------------------------------------------------
// C-ABI
extern "C" {

int ghmm_load(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) return 0;
    for (int d = 0; d < n; d++) {
        cudaDeviceProp p;
        if (cudaGetDeviceProperties(&p, d) == cudaSuccess && p.major == 10 && p.minor == 3) return 1;
    }
    return 0;
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
    const int mk = t->max_rows_per_lane ? t->max_rows_per_lane : kMaxK32;
    const int mm = t->max_rows_per_lane_multi ? t->max_rows_per_lane_multi : kMaxK32;
    const int cc = t->chunk_cols ? t->chunk_cols : 16384;
    if (mk < 1 || mk > kMaxK32 || mm < 1 || mm > kMaxK32 || cc < 1)
        return fail(ctx, GHMM_ERR_ARG, "tuning out of range (rows per lane 1..8, chunk_cols >= 1)");
    ctx->max_k = mk;
    ctx->max_k_multi = mm;
    ctx->chunk_cols = cc;
    return GHMM_OK;
}

int ghmm_done(ghmm_ctx *ctx) {
    if (!ctx) return GHMM_ERR_STATE;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    ctx->scratch_batch.release();
    ctx->calib_scratch.release();
    ctx->calib_flags.release();
    ctx->calib_ones.release();
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
    Source src;
    src.regions = regions;
    src.n_regions = n_regions;
    ghmm_batch &b = ctx->scratch_batch;
    int rc = batch_marshal(ctx, src, b);
    if (!rc) rc = batch_upload(ctx, b);
    if (!rc) rc = batch_forward(ctx, b, ctx->double_precision ? GHMM_MODE_FP64 : GHMM_MODE_FP32_RERUN);
    if (!rc) rc = batch_results(ctx, b, out);
    return rc;
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
    if (!rc) rc = batch_upload(ctx, *b);
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
    if (!rc) rc = batch_upload(ctx, *b);
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
    if (mode < 0 || mode > 2) return fail(ctx, GHMM_ERR_ARG, "unknown mode");
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
    st->n_rerun = b->last_mode == GHMM_MODE_FP32_RERUN ? b->last_rerun : 0;
    st->n_fp64_direct = b->last_mode == GHMM_MODE_FP64 ? b->n_direct_fp64mode : b->n_direct;
    st->n_tasks_fp32 = b->n_tasks;
    st->n_launches = b->last_launches;
    st->reserved = 0;
    st->ms_fp32 = b->ms_fp32;
    st->ms_fp64 = b->ms_fp64;
    st->ms_plain = b->ms_plain;
    st->ms_total = b->ms_total;
    st->h2d_bytes = b->upload_bytes + b->forward_h2d;
    st->d2h_bytes = b->forward_d2h + b->results_d2h;
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
    Source src;
    src.flat = flat;
    src.n_regions = flat->n_regions;
    ghmm_batch &b = ctx->scratch_batch;
    int rc = batch_marshal(ctx, src, b);
    if (!rc) rc = batch_upload(ctx, b);
    if (!rc) rc = batch_forward(ctx, b, ctx->double_precision ? GHMM_MODE_FP64 : GHMM_MODE_FP32_RERUN);
    if (!rc) rc = batch_results(ctx, b, out);
    return rc;
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
