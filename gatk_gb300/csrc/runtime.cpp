// runtime.cpp -- the context behind the C-ABI (include/ghmm.h) and the entry points that are neither batch
// internals (batch.cpp), queues (queue.cpp), PD-HMM (pd_host.cpp) nor raw reads (raw_host.cpp): loading and
// initialising, tuning and the autotuner, batch handles, statistics, the post-likelihood step, calibration, peaks.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "runtime_internal.h"

namespace ghmm {
std::atomic<int64_t> g_refuse_allocations{0};
}

namespace {

std::mutex g_init_error_mu;
std::string g_init_error;

}  // namespace

namespace ghmm {
namespace rt {


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


}  // namespace rt
}  // namespace ghmm

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
    ctx->tables.lm2m_d = dt->lm2m;
    ctx->alive = true;
    *out = ctx;
    return GHMM_OK;
}

// Bytes of per-warp calibration scratch one call may hold: GHMM_CALIB_SCRATCH_BYTES, else 4 GiB.
static int64_t calib_scratch_budget() {
    const char *v = std::getenv("GHMM_CALIB_SCRATCH_BYTES");
    if (v && *v) {
        char *end = nullptr;
        const long long b = std::strtoll(v, &end, 10);
        if (end && *end == 0 && b > 0) return (int64_t)b;
    }
    return (int64_t)4 << 30;
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
    if (in->max_read_len < 1 || in->max_read_len > kCalibMaxRead)
        return fail(ctx, GHMM_ERR_ARG, "calibration supports reads of 1..65536 bases (max_read_len)");
    if (in->max_hap_len < 1) return fail(ctx, GHMM_ERR_ARG, "max_hap_len must be >= 1");
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    // one strip of 32 k rows up to 256 bases, strips of 256 rows (k = 8) beyond
    const int k = std::min((in->max_read_len + 31) / 32, 8);
    // the backward keeps checkpoints in per-warp scratch, and a read of several strips passes each strip's last
    // row through it in the forward too
    const bool strips = in->max_read_len > 32 * 8;
    const int64_t per_warp = calib_scratch_per_warp(k, in->max_hap_len, in->max_read_len, true);  // sized for FP64
    const int64_t warps_per_block = calib_block() / 32;
    int64_t blocks = calib_grid(ctx->sm_count);
    if (backward || strips) {
        // fewer warps (each taking more pairs) where long pairs would make a full grid's scratch exceed the budget
        const int64_t budget = calib_scratch_budget();
        blocks = std::max<int64_t>(1, std::min(blocks, budget / (per_warp * warps_per_block)));
        GHMM_CUDA(ctx->calib_scratch.reserve((size_t)(per_warp * warps_per_block * blocks)), "calibration scratch");
    }
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
                             calib_scratch_per_warp(k, in->max_hap_len, in->max_read_len, false), loglik, weights,
                             gopen, gcont, flags, (int)blocks, ctx->sm_count, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "calibration FP32 launch");
    }
    int e = launch_calib(ctx->tables, *in, k, backward, true, ctx->calib_scratch.p, per_warp, loglik, weights, gopen,
                         gcont, flags, (int)blocks, ctx->sm_count, s);
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
    for (auto &pb : ctx->pd_batch) pb.release();
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
    if (ctx->pd_stream2) cudaStreamDestroy(ctx->pd_stream2);
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

