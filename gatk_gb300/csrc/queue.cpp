// queue.cpp -- the streaming queue (ghmm_queue_*) and the pipeline of batches that large synchronous calls run as.
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

#include "runtime_internal.h"

namespace ghmm {
namespace rt {


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
    if (q->serial_fp32) {  // the FP32 pass after the other slot's (its FP64 reruns and copies still overlap)
        const int o = 1 - i;
        if (q->inflight[o] && q->slot[o].events_ready)
            GHMM_CUDA(cudaStreamWaitEvent(q->stream[i], q->slot[o].ev[2], 0), "wait for the previous FP32 pass");
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
int queue_open(ghmm_ctx *ctx, int64_t batch_cells, ghmm_queue **out, const ghmm_read_prep *raw_prep,
               const RouteBound *bound) {
    auto *q = new ghmm_queue();
    q->ctx = ctx;
    q->batch_cells = batch_cells > 0 ? batch_cells : (int64_t)2e11;
    // a streaming queue's batches run their FP32 passes in turn (workload 4 through the queue, 30,000 regions in
    // batches of 2e11 cells: 3,848 against 3,698 GCUPS side by side)
    q->serial_fp32 = true;
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


// Raw reads (mapq non-NULL, src.regions over the raw view's reads): every batch gets the read preparation prep on
// the device after its upload.
// Region cuts [0 = c_0 < c_1 < ... = G] of a pipelined call over regions of the given cells.  Below 5e11 cells: three
// chunks, after 1/8 and 1/2 of the cells, because each chunk's launches, graph capture and kernel tails cost a fixed
// time (workload 1 end to end through ghmm_compute_regions: 95.6 ms against 101.5 ms for the finer cut at 3,000
// regions; the regular calls run below 1.5e11 cells as one batch, the one-shot PD-HMM calls in chunks down to 8
// regions, which gain or lose nothing measurable against one chunk at 1,000 regions).  Above: 1/16 of the cells first, each next chunk 2.5 times the last up to
// 1/3, so the first marshal the device waits for stays short (281.5 ms against 285.8 ms for three chunks at 10,000
// regions).  No cut leaves fewer than 8 regions behind it.
std::vector<int64_t> pipeline_cuts(const std::vector<int64_t> &cells) {
    const int64_t G = (int64_t)cells.size();
    int64_t total = 0;
    for (int64_t c : cells) total += c;
    std::vector<int64_t> cut{0};
    if (total < kPipelineLargeCells) {
        const int64_t marks[2] = {total / 8, total / 2};
        int64_t c = 0;
        int m = 0;
        for (int64_t g = 0; g < G && m < 2; g++) {
            c += cells[(size_t)g];
            if (c >= marks[m] && G - g - 1 >= 8) {
                cut.push_back(g + 1);
                m++;
            }
        }
        cut.push_back(G);
        return cut;
    }
    int64_t target = std::max<int64_t>(total / 16, 1);
    for (int64_t g0 = 0; g0 < G;) {
        int64_t g1 = g0, c = 0;
        while (g1 < G && (c < target || g1 == g0)) c += cells[(size_t)g1++];
        if (G - g1 < 8) g1 = G;
        cut.push_back(g1);
        target = std::min(target * 5 / 2, std::max<int64_t>(total / 3, 1));
        g0 = g1;
    }
    return cut;
}

int pipelined_compute(ghmm_ctx *ctx, const Source &src, const std::vector<int64_t> &reg_cells,
                      const std::vector<int64_t> &reg_out, double *out, const int32_t *mapq,
                      int32_t max_len, const ghmm_read_prep *prep, const RouteBound *bound) {
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
        // the large schedule's chunks run their FP32 passes in turn: bucket kernels of two such chunks side by side
        // ran slower than one after the other (workload 1 end to end at 10,000 regions: 290 against 282 ms), while the
        // small schedule's chunks gain from filling each other's kernel tails (42.4 against 44.5 ms at 1,000 regions)
        int64_t total = 0;
        for (int64_t c : reg_cells) total += c;
        q->serial_fp32 = total >= kPipelineLargeCells;
    }
    const int64_t G = src.n_regions;
    std::vector<int64_t> first_read;  // raw reads: the batch's reads' mapping qualities go with the batch
    if (mapq) {
        first_read.assign((size_t)G + 1, 0);
        for (int64_t g = 0; g < G; g++) first_read[(size_t)g + 1] = first_read[(size_t)g] + src.regions[g].n_reads;
    }
    const std::vector<int64_t> cut = pipeline_cuts(reg_cells);
    for (size_t i = 0; i + 1 < cut.size(); i++) {
        const int64_t g0 = cut[i], g1 = cut[i + 1];
        int64_t c = 0;
        for (int64_t g = g0; g < g1; g++) c += reg_cells[(size_t)g];
        auto u = borrowed_unit(src, g0, g1, out + reg_out[(size_t)g0], reg_out[(size_t)g1] - reg_out[(size_t)g0], c);
        if (mapq) {
            u->mapq.assign(mapq + first_read[(size_t)g0], mapq + first_read[(size_t)g1]);
            u->max_len = max_len;
        }
        queue_submit(q, std::move(u));
    }
    int rc = queue_wait_all(q);
    {
        std::lock_guard<std::mutex> lk(q->mu);
        queue_set_raw(q, nullptr, nullptr);
    }
    if (rc) return queue_status(q);
    return GHMM_OK;
}

// Per-region cells and output offsets of a region array or flat input; false if a count is negative or a region's
// array is NULL.  The counts are checked in region order first (nothing past the first bad region is read); then a
// region array's read and haplotype lengths are summed with the regions in parallel.
bool region_sizes(const Source &src, std::vector<int64_t> &cells, std::vector<int64_t> &outo, int threads) {
    const int64_t G = src.n_regions;
    cells.assign((size_t)G, 0);
    outo.assign((size_t)G + 1, 0);
    for (int64_t g = 0; g < G; g++) {
        int64_t nr, nh;
        if (src.flat) {
            const ghmm_flat *f = src.flat;
            nr = f->region_read_off[g + 1] - f->region_read_off[g];
            nh = f->region_hap_off[g + 1] - f->region_hap_off[g];
            if (nr < 0 || nh < 0) return false;
        } else {
            const ghmm_region &rg = src.regions[g];
            nr = rg.n_reads;
            nh = rg.n_haps;
            if (nr < 0 || nh < 0 || (nr > 0 && !rg.reads) || (nh > 0 && !rg.haps)) return false;
        }
        outo[(size_t)g + 1] = outo[(size_t)g] + nr * nh;
    }
    parallel_for(G, src.flat ? 1 : threads, [&](int64_t g) {
        int64_t sr = 0, sh = 0;
        if (src.flat) {
            const ghmm_flat *f = src.flat;
            sr = f->read_off[f->region_read_off[g + 1]] - f->read_off[f->region_read_off[g]];
            sh = f->hap_off[f->region_hap_off[g + 1]] - f->hap_off[f->region_hap_off[g]];
        } else {
            const ghmm_region &rg = src.regions[g];
            for (int32_t r = 0; r < rg.n_reads; r++) sr += std::max(rg.reads[r].length, 0);
            for (int32_t h = 0; h < rg.n_haps; h++) sh += std::max(rg.haps[h].length, 0);
        }
        cells[(size_t)g] = sr * sh;
    });
    return true;
}

// Synchronous compute of regions or flat input: one batch for small inputs, the pipeline for large ones.
int compute_sync(ghmm_ctx *ctx, const Source &src, double *out) {
    std::vector<int64_t> cells, outo;
    if (!region_sizes(src, cells, outo, hw_threads(ctx->max_threads)))
        return fail(ctx, GHMM_ERR_ARG, "negative count or NULL array in a region");
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


}  // namespace rt
}  // namespace ghmm

extern "C" {

int ghmm_debug_pipeline_cuts(const int64_t *cells, int64_t n_regions, int64_t *cuts, int64_t cap, int64_t *n_cuts) {
    if (n_regions < 0 || (n_regions > 0 && !cells) || cap < 0 || (cap > 0 && !cuts) || !n_cuts) return GHMM_ERR_ARG;
    for (int64_t g = 0; g < n_regions; g++)
        if (cells[g] < 0) return GHMM_ERR_ARG;
    const std::vector<int64_t> cut = pipeline_cuts(std::vector<int64_t>(cells, cells + n_regions));
    *n_cuts = (int64_t)cut.size();
    for (int64_t i = 0; i < std::min<int64_t>(cap, (int64_t)cut.size()); i++) cuts[i] = cut[(size_t)i];
    return GHMM_OK;
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


}  // extern "C"
