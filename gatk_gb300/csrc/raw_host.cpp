// raw_host.cpp -- raw reads (ghmm_*_raw): the checks and views of raw reads, and the read preparation on the device
// (prep.cu) after a batch's upload.
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

// -------------------------------------------------------------------------------------------------
// Raw reads: the regular marshal over the reads' bases and raw qualities (45 where a read has no BI / BD tag, the
// constant gap continuation penalty), then prep.cu rewrites the quality planes on the device.  The host's routing
// checks see the raw qualities; a read whose prepared qualities would make the FP32 or rescaled FP64 forms
// overflow still ends up exact, because a non-finite sum sends its pair on to the next tier.



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
    });
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
    v.reads.reset(new ghmm_read[(size_t)std::max<int64_t>(first[(size_t)G], 1)]);
    v.mapq.resize((size_t)first[(size_t)G]);
    parallel_for(G, threads, [&](int64_t g) {
        const ghmm_raw_region &rg = raw[g];
        ghmm_read *rr = v.reads.get() + first[(size_t)g];
        int32_t *mq = v.mapq.data() + first[(size_t)g];
        for (int32_t r = 0; r < rg.n_reads; r++) {
            const ghmm_raw_read &rd = rg.reads[r];
            rr[r] = ghmm_read{rd.bases, rd.quals, rd.ins_quals ? rd.ins_quals : v.q45.data(),
                              rd.del_quals ? rd.del_quals : v.q45.data(), v.qgcp.data(), rd.length};
            mq[r] = rd.mapping_quality;
        }
        v.regions[(size_t)g] = ghmm_region{rr, rg.n_reads, rg.haps, rg.n_haps};
    });
    return GHMM_OK;
}


int raw_prepare_device(ghmm_ctx *ctx, ghmm_batch &b, const int32_t *mapq, int32_t max_len,
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
    // the gap penalties changed: the FP32 pass's per-read scale again
    const int e2 = launch_read_scale(ctx->tables, b.dev, NR, b.d_read_scale.p, ctx->sm_count, s);
    if (e2) return cuda_fail(ctx, (cudaError_t)e2, "read scale launch");
    b.prep_timed = true;
    b.upload_bytes += NR * 4;
    return GHMM_OK;
}

}  // namespace rt
}  // namespace ghmm

extern "C" {

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
        if (!region_sizes(src, cells, outo, hw_threads(ctx->max_threads)))
            return fail(ctx, GHMM_ERR_ARG, "negative count or NULL array in a region");
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


}  // extern "C"
