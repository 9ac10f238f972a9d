// pd_host.cpp -- PD-HMM batches on the host side (ghmm_pd_*): the regular marshal over the haplotypes' bases plus
// the PD flag and HMM state planes, and the forward through pd.cu.
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
#include <functional>
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
// PD-HMM batches: the regular marshal over the haplotypes' bases, plus per haplotype column the PD flags and the
// HMM state codes (PdPlanes), and a forward that runs every pair through pd.cu.


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


// Whether the packed FP32 kernel (pd_packed.cu) can take a haplotype: its row-end state is not INSIDE_DEL.  Row 1
// starts NORMAL and the later rows start in the previous row's end state; an AFTER_DEL there changes nothing (the
// first column's inputs from column 0 are zero in every row below row 1, branch states included), so every row
// sees one state sequence, while an open INSIDE_DEL keeps the later rows' branch states where row 1 renews them.
static bool pd_packable(const uint8_t *f, int H) {
    int st = 0;
    for (int j = 0; j < H; j++) {
        if (st == 2) st = 0;
        if (f[j] & 2) st = 1;
        if (f[j] & 4) st = 2;
    }
    return st != 1;
}

// The packed kernel's op byte of every column of one haplotype (pd_packed.cu), from its flags f, its bytes y and the
// state codes of pd_states (bits 2-3: the state of rows >= 2, equal to the first row's for a packable haplotype).
// A column's branch state is needed when the next column is AFTER_DEL (it reads it), when the next column is
// INSIDE_DEL and needs its own (it keeps it), or when the column ends a deletion (the row below's I reads it); only
// then does a NORMAL or AFTER_DEL column store it (kPdOpCopy).  An
// SNP column whose alternatives and base cover all four bases gets the column code of N in code (the column-code
// plane), which matches every read base as isBasePDMatching then does.
static void pd_ops(const uint8_t *f, const uint8_t *y, const uint8_t *states, int H, uint8_t *op, uint8_t *code) {
    bool need_next = false;
    for (int j = H - 1; j >= 0; --j) {
        const int st = (states[j] >> 2) & 3;
        const int st_next = j + 1 < H ? (states[j + 1] >> 2) & 3 : 0;
        const bool del_end = (f[j] & 4) != 0;
        const bool need = st_next == 2 || (st_next == 1 && need_next) || del_end;
        uint32_t o = 0;
        if (st != 1 && need) o |= kPdOpCopy;  // (INSIDE_DEL keeps the branch state it has)
        if (st == 2 && j > 0) o |= kPdOpAfter;  // (at the first column AFTER_DEL acts as NORMAL, pd_packable)
        if (del_end) o |= kPdOpDelEnd;
        if (st_next == 2) o |= kPdOpNextAfter;
        const int ref = base_index(y[j]);
        const int alts = (f[j] >> 3) & 15;
        if ((f[j] & 1) && ref < 4 && (alts & ~(1 << ref))) {  // (an N column matches every read base already)
            const int match = alts | (1 << ref);  // bases A, C, G, T = bits 0..3 that match the column
            const int n = ((match >> 0) & 1) + ((match >> 1) & 1) + ((match >> 2) & 1) + ((match >> 3) & 1);
            if (n == 4) {
                code[j] = (uint8_t)((code[j] & ~7u) | 4u);
            } else if (n == 3) {
                int u = 0;
                while ((match >> u) & 1) ++u;
                o |= kPdOpSnp | kPdOpSnpAllBut | ((uint32_t)u << kPdOpAltShift);
            } else {
                int alt = 0;
                while (!((alts >> alt) & 1) || alt == ref) ++alt;
                o |= kPdOpSnp | ((uint32_t)alt << kPdOpAltShift);
            }
        }
        op[j] = (uint8_t)o;
        need_next = need;
    }
}

int pd_marshal(ghmm_ctx *ctx, const ghmm_pd_region *regs, int64_t G, ghmm_batch &b, const RouteBound *bound) {
    std::vector<ghmm_region> rr((size_t)G);
    std::vector<std::vector<ghmm_hap>> hh((size_t)G);
    std::vector<const uint8_t *> pdp;
    std::vector<uint8_t> region_direct((size_t)G, 0);
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
    parallel_for(G, hw_threads(ctx->max_threads), [&](int64_t g) {
        for (int32_t h = 0; h < regs[g].n_haps; h++) {
            const ghmm_pd_hap &hp = regs[g].haps[h];
            if (hp.length > 0 && !pd_packable(hp.pd_bases, hp.length)) {
                region_direct[(size_t)g] = 1;
                break;
            }
        }
    });
    Source src;
    src.regions = rr.data();
    src.n_regions = G;
    src.bound = bound;
    src.region_direct = region_direct.data();
    int rc = batch_marshal(ctx, src, b);
    if (rc) return rc;
    const int64_t NH = b.n_haps, HB = b.hap_bytes;
    // flags | states | kCodePad zeros | ops | kCodePad zeros
    const int64_t pd_bytes = 3 * HB + 2 * kCodePad;
    GHMM_CUDA(b.h_pd.reserve((size_t)pd_bytes), "pinned PD planes");
    const int64_t *o = b.h_off.p;
    const int64_t *hap_off = o + b.n_reads + 1;
    uint8_t *flags = b.h_pd.p, *states = b.h_pd.p + HB, *ops = b.h_pd.p + 2 * HB + kCodePad;
    memset(ops - kCodePad, 0, (size_t)kCodePad);
    memset(ops + HB, 0, (size_t)kCodePad);
    const uint8_t *hraw = b.h_hap.p;
    uint8_t *hcode = b.h_hap.p + HB + kCodePad;
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
        pd_ops(flags + a, hraw + a, code, H, ops + a, hcode + a);
    });
    // a read base outside ACGTacgtN that meets an undetermined SNP column throws in the reference
    const int64_t *rro = o + b.n_reads + 1 + NH + 1, *rho = rro + G + 1;
    const uint8_t *bases = b.h_planes.p;
    std::atomic<bool> unexpected{false};
    parallel_for(G, hw_threads(ctx->max_threads), [&](int64_t g) {
        for (int64_t i = o[rro[g]]; i < o[rro[g + 1]]; i++) {
            const uint8_t x = bases[i];
            if (pd_read_base_ok(x)) continue;
            for (int64_t h = rho[g]; h < rho[g + 1]; h++)
                for (int64_t j = hap_off[h]; j < hap_off[h + 1]; j++)
                    if ((flags[j] & 1) && hraw[j] != x && hraw[j] != 'N') unexpected = true;
        }
    });
    if (unexpected) return fail(ctx, GHMM_ERR_ARG, "Found unexpected base in alt alleles");
    b.has_pd = true;
    return GHMM_OK;
}

int pd_upload(ghmm_ctx *ctx, ghmm_batch &b, cudaStream_t s) {
    int rc = batch_upload(ctx, b, s);
    if (rc) return rc;
    const int64_t HB = b.hap_bytes, pd_bytes = 3 * HB + 2 * kCodePad;
    GHMM_CUDA(b.d_pd.reserve((size_t)pd_bytes), "device PD planes");
    GHMM_CUDA(cudaMemcpyAsync(b.d_pd.p, b.h_pd.p, (size_t)pd_bytes, cudaMemcpyHostToDevice, s), "H2D PD planes");
    b.pd.flags = b.d_pd.p;
    b.pd.states = b.d_pd.p + HB;
    b.pd.ops = b.d_pd.p + 2 * HB + kCodePad;
    b.upload_bytes += pd_bytes;
    return GHMM_OK;
}

// fp32: the read-pair tasks of the regular marshal through the packed FP32 kernel (pd_packed.cu) and the pairs without
// a task through the general FP32 one (pd.cu), then the pairs whose FP32 sums underflow in the FP64 one (K = 4);
// otherwise every pair in FP64
int batch_forward_pd(ghmm_ctx *ctx, ghmm_batch &b, bool fp32) {
    const int rc = pd_forward_enqueue(ctx, b, fp32, ctx->stream);
    return rc ? rc : pd_forward_finish(ctx, b);
}

// The kernels of one PD forward on stream s, and the D2H of its counters, without waiting (pd_forward_finish waits).
int pd_forward_enqueue(ghmm_ctx *ctx, ghmm_batch &b, bool fp32, cudaStream_t s) {
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    // the general kernel's pairs (FP64: every pair; FP32: those without a task), grouped by the rows per lane K of the
    // read (the strip height 32 K, K = 1..4, that needs the fewest rows; ties to the larger K, i.e. fewer strips), in
    // region order within a group
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
    auto for_each_pair = [&](auto fn) {
        if (fp32) {
            const int64_t n = b.n_direct + b.n_direct_exact;
            for (int64_t i = 0; i < n; i++) fn(b.h_direct.p[i]);
        } else {
            for (int64_t g = 0; g < b.n_regions; g++)
                for (int64_t r = rro[g]; r < rro[g + 1]; r++)
                    for (int64_t h = rho[g]; h < rho[g + 1]; h++) fn(PairRef{(int32_t)r, (int32_t)h});
        }
    };
    int64_t kcount[kPdMaxK32 + 1] = {0};
    for_each_pair([&](const PairRef &p) { kcount[pick_k(o[p.read + 1] - o[p.read])]++; });
    int64_t kbegin[kPdMaxK32 + 2] = {0};
    for (int kk = 1; kk <= maxk; kk++) kbegin[kk + 1] = kbegin[kk] + kcount[kk];
    int64_t kpos[kPdMaxK32 + 1];
    for (int kk = 1; kk <= maxk; kk++) kpos[kk] = kbegin[kk];
    for_each_pair([&](const PairRef &p) { b.h_fp64all.p[kpos[pick_k(o[p.read + 1] - o[p.read])]++] = p; });
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
    const bool packed = fp32 && b.n_tasks > 0;
    if (packed)
        for (auto &bk : b.buckets) {
            hc[kNumCounters + bk.key] = bk.begin;
            hc[kNumCounters + kNumBucketKeys + bk.key] = bk.count;
        }
    GHMM_CUDA(cudaMemcpyAsync(b.d_counters.p, hc, (kNumCounters + 2 * kNumBucketKeys) * sizeof(int32_t),
                              cudaMemcpyHostToDevice, s), "H2D counters");
    b.h_nout.p[0] = b.n_out;
    if (packed)
        GHMM_CUDA(cudaMemcpyAsync(b.d_nout.p, b.h_nout.p, sizeof(int64_t), cudaMemcpyHostToDevice, s),
                  "H2D output count");
    GHMM_CUDA(cudaEventRecord(b.ev[1], s), "event");
    int launches = 0;
    if (packed) {  // read-pair tasks, then the log10 epilogue of their sums (before the kernels that write log10)
        for (auto &bk : b.buckets) {
            int bp = 0;
            if (pd_bucket_occupancy(bk.key, &bp) != 0 || bp <= 0) bp = 1;
            const int64_t want = (bk.count + kWarpsPerBlock - 1) / kWarpsPerBlock;
            int g = (int)std::max<int64_t>(1, std::min<int64_t>(want, (int64_t)ctx->sm_count * bp));
            if (bk.key & 16) g = std::min(g, bk.grid);  // the strip scratch is sized for the regular kernel's grid
            int e = launch_pd_bucket(ctx->tables, b.dev, b.pd.ops, bk.key, g, s);
            if (e) return cuda_fail(ctx, (cudaError_t)e, "PD-HMM packed launch");
            launches++;
        }
        int e = launch_finalize_fp32(b.dev.out, b.dev.n_out_dev, ctx->sm_count, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "PD-HMM FP32 finalize launch");
        launches++;
    }
    for (int kk = maxk; kk >= 1; --kk) {  // longest strips first
        if (kcount[kk] == 0) continue;
        const int cursor = (fp32 ? kCounterPdF32Base : kCounterPdBase) + kk;
        int e = launch_pd(ctx->tables, b.dev, b.pd, kk, fp32, (int)kbegin[kk], (int)kcount[kk], cursor, nullptr, grid, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "PD-HMM launch");
        launches++;
    }
    GHMM_CUDA(cudaEventRecord(b.ev[4], s), "event");
    if (fp32) {  // the FP32 pass's underflows, queued at rerun[capacity..), in FP64
        int e = launch_pd(ctx->tables, b.dev, b.pd, kPdMaxK, false, (int)b.dev.rerun_capacity, 0,
                          kCounterPdRerunCursor, b.d_counters.p + kCounterPdRerun, grid, s);
        if (e) return cuda_fail(ctx, (cudaError_t)e, "PD-HMM FP64 rerun launch");
        launches++;
    }
    GHMM_CUDA(cudaEventRecord(b.ev[2], s), "event");
    GHMM_CUDA(cudaMemcpyAsync(hc, b.d_counters.p, kNumCounters * sizeof(int32_t), cudaMemcpyDeviceToHost, s),
              "D2H counters");
    GHMM_CUDA(cudaEventRecord(b.ev[3], s), "event");
    b.last_mode = fp32 ? GHMM_MODE_PD_FP32 : GHMM_MODE_PD;
    b.last_launches = launches;
    b.forward_h2d = k * (int64_t)sizeof(PairRef) + (kNumCounters + 2 * kNumBucketKeys) * 4 + (packed ? 8 : 0);
    b.forward_d2h = kNumCounters * 4;
    return GHMM_OK;
}

int pd_forward_finish(ghmm_ctx *ctx, ghmm_batch &b) {
    GHMM_CUDA(cudaEventSynchronize(b.ev[3]), "PD-HMM kernel");
    const bool fp32 = b.last_mode == GHMM_MODE_PD_FP32;
    float ms = 0, ms_a = 0, ms_b = 0;
    cudaEventElapsedTime(&ms_a, b.ev[1], b.ev[4]);
    cudaEventElapsedTime(&ms_b, b.ev[4], b.ev[2]);
    b.ms_fp32 = fp32 ? ms_a : 0;
    b.ms_fp64 = fp32 ? ms_b : ms_a + ms_b;
    b.ms_plain = 0;
    cudaEventElapsedTime(&ms, b.ev[0], b.ev[3]);
    b.ms_total = ms;
    const int32_t *hc = b.h_counters.p;
    b.last_rerun = fp32 ? hc[kCounterPdRerun] : 0;
    b.last_exact = 0;
    if (hc[3] == 1) return fail(ctx, GHMM_ERR_CUDA, "PD-HMM FP64 rerun queue overflow");
    if (hc[3] != 0) return fail(ctx, GHMM_ERR_CUDA, "device-side scratch bound exceeded");
    return GHMM_OK;
}


// The one-shot PD-HMM calls in chunks of regions, pipelined on two streams: chunk i+1 is marshalled on the host and
// enqueued (upload, preparation, forward) on the other slot's stream while chunk i runs, so its kernels start as
// chunk i's last tasks leave SMs free; then chunk i's results are read.  Chunks as pipeline_cuts cuts them (below
// 5e11 cells three, of 1/8, 3/8 and 1/2 of the cells: on 1,000 regions of workload 1 with PD flags, 85 ms a call
// against 112 ms for the finer cut of large inputs and 84 ms unchunked; on 3,000 regions, 198 ms against 209 ms and
// 232 ms).  host(g0, g1, slot) stages regions [g0, g1) in ctx->pd_batch[slot]; device(slot, stream) uploads it (and
// prepares raw reads).
int pd_pipelined(ghmm_ctx *ctx, const std::vector<int64_t> &cells, const std::vector<int64_t> &outo, double *out,
                 const std::function<int(int64_t, int64_t, int)> &host,
                 const std::function<int(int, cudaStream_t)> &device) {
    const std::vector<int64_t> cut = pipeline_cuts(cells);
    if (!ctx->pd_stream2)
        GHMM_CUDA(cudaStreamCreateWithFlags(&ctx->pd_stream2, cudaStreamNonBlocking), "cudaStreamCreate");
    const cudaStream_t streams[2] = {ctx->stream, ctx->pd_stream2};
    const bool fp32 = !ctx->double_precision;
    auto start = [&](size_t i) {
        const int slot = (int)(i & 1);
        int rc = host(cut[i], cut[i + 1], slot);
        if (!rc) rc = device(slot, streams[slot]);
        if (!rc) rc = pd_forward_enqueue(ctx, ctx->pd_batch[slot], fp32, streams[slot]);
        return rc;
    };
    int rc = start(0);
    for (size_t i = 0; !rc && i + 1 < cut.size(); i++) {
        const int slot = (int)(i & 1);
        const int rc_next = i + 2 < cut.size() ? start(i + 1) : GHMM_OK;
        ghmm_batch &b = ctx->pd_batch[slot];
        rc = pd_forward_finish(ctx, b);
        if (!rc) rc = batch_results_on(ctx, b, out + outo[(size_t)cut[i]], streams[slot]);
        if (!rc) rc = rc_next;
    }
    // nothing of this call may still run on either stream when it returns
    cudaStreamSynchronize(streams[0]);
    cudaStreamSynchronize(streams[1]);
    return rc;
}

// PD regions of raw reads: the raw reads' view (checks, 45s and the constant GCP) as the regular raw path builds it,
// then the PD marshal over it, the upload, and the read preparation on the device.
int pd_raw_build(ghmm_ctx *ctx, const ghmm_pd_raw_region *regions, int32_t n_regions, const ghmm_read_prep *prep,
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
    rc = pd_marshal(ctx, pr.data(), n_regions, b, v.has_bound ? &v.bound : nullptr);
    if (!rc) rc = pd_upload(ctx, b, ctx->stream);
    if (!rc) rc = raw_prepare_device(ctx, b, v.mapq.data(), v.max_len, prep, ctx->stream);
    return rc;
}



}  // namespace rt
}  // namespace ghmm

extern "C" {

int ghmm_debug_pd_ops(const uint8_t *bases, const uint8_t *pd_flags, int32_t H, uint8_t *ops, uint8_t *codes) {
    if (H < 0 || (H > 0 && (!bases || !pd_flags || !ops || !codes))) return GHMM_ERR_ARG;
    std::vector<uint8_t> st((size_t)H, 0);
    const int end1 = pd_states(pd_flags, H, 0, st.data(), 0);
    pd_states(pd_flags, H, end1, st.data(), 2);
    for (int32_t j = 0; j < H; j++) {
        if (pd_flags[j] & 4) st[(size_t)j] |= 16;
        codes[j] = base_index(bases[j]);
    }
    pd_ops(pd_flags, bases, st.data(), H, ops, codes);
    return pd_packable(pd_flags, H) ? 1 : 0;
}

int ghmm_pd_batch_create(ghmm_ctx *ctx, const ghmm_pd_region *regions, int32_t n_regions, ghmm_batch **out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (!out || n_regions < 0 || (n_regions > 0 && !regions)) return fail(ctx, GHMM_ERR_ARG, "bad arguments");
    GHMM_CUDA(cudaSetDevice(ctx->device), "cudaSetDevice");
    auto *b = new ghmm_batch();
    int rc = pd_marshal(ctx, regions, n_regions, *b, nullptr);
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
    std::vector<int64_t> cells((size_t)n_regions, 0), outo((size_t)n_regions + 1, 0);
    for (int32_t g = 0; g < n_regions; g++) {
        const ghmm_pd_region &rg = regions[g];
        if (rg.n_reads < 0 || rg.n_haps < 0 || (rg.n_reads > 0 && !rg.reads) || (rg.n_haps > 0 && !rg.haps))
            return fail(ctx, GHMM_ERR_ARG, "bad PD region");
        int64_t sr = 0, sh = 0;
        for (int32_t r = 0; r < rg.n_reads; r++) sr += std::max(rg.reads[r].length, 0);
        for (int32_t h = 0; h < rg.n_haps; h++) sh += std::max(rg.haps[h].length, 0);
        cells[(size_t)g] = sr * sh;
        outo[(size_t)g + 1] = outo[(size_t)g] + (int64_t)rg.n_reads * rg.n_haps;
    }
    return pd_pipelined(
        ctx, cells, outo, out,
        [&](int64_t g0, int64_t g1, int slot) {
            return pd_marshal(ctx, regions + g0, g1 - g0, ctx->pd_batch[slot], nullptr);
        },
        [&](int slot, cudaStream_t st) { return pd_upload(ctx, ctx->pd_batch[slot], st); });
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
    std::vector<int64_t> cells((size_t)n_regions, 0), outo((size_t)n_regions + 1, 0);
    for (int32_t g = 0; g < n_regions; g++) {
        const ghmm_pd_raw_region &rg = regions[g];
        if (rg.n_reads < 0 || rg.n_haps < 0 || (rg.n_reads > 0 && !rg.reads) || (rg.n_haps > 0 && !rg.haps))
            return fail(ctx, GHMM_ERR_ARG, "bad PD region");
        int64_t sr = 0, sh = 0;
        for (int32_t r = 0; r < rg.n_reads; r++) sr += std::max(rg.reads[r].length, 0);
        for (int32_t h = 0; h < rg.n_haps; h++) sh += std::max(rg.haps[h].length, 0);
        cells[(size_t)g] = sr * sh;
        outo[(size_t)g + 1] = outo[(size_t)g] + (int64_t)rg.n_reads * rg.n_haps;
    }
    // the raw view of each slot's chunk (its mapping qualities) lives until that chunk's preparation has read them
    RawView views[2];
    return pd_pipelined(
        ctx, cells, outo, out,
        [&](int64_t g0, int64_t g1, int slot) {
            RawView &v = views[slot];
            v = RawView();
            std::vector<ghmm_raw_region> rr((size_t)(g1 - g0));
            for (int64_t g = g0; g < g1; g++)
                rr[(size_t)(g - g0)] = ghmm_raw_region{regions[g].reads, regions[g].n_reads, nullptr, 0};
            int rc = raw_view(ctx, rr.data(), g1 - g0, prep, v);
            if (rc) return rc;
            std::vector<ghmm_pd_region> pr((size_t)(g1 - g0));
            for (int64_t g = g0; g < g1; g++)
                pr[(size_t)(g - g0)] = ghmm_pd_region{v.regions[(size_t)(g - g0)].reads, regions[g].n_reads,
                                                      regions[g].haps, regions[g].n_haps};
            return pd_marshal(ctx, pr.data(), g1 - g0, ctx->pd_batch[slot], v.has_bound ? &v.bound : nullptr);
        },
        [&](int slot, cudaStream_t st) {
            ghmm_batch &b = ctx->pd_batch[slot];
            int rc = pd_upload(ctx, b, st);
            if (!rc) rc = raw_prepare_device(ctx, b, views[slot].mapq.data(), views[slot].max_len, prep, st);
            return rc;
        });
}

int ghmm_pd_compute_likelihoods(ghmm_ctx *ctx, const ghmm_read *reads, int32_t n_reads, const ghmm_pd_hap *haps,
                                int32_t n_haps, double *out) {
    if (!ctx || !ctx->alive) return GHMM_ERR_STATE;
    if (n_reads == 0 || n_haps == 0) return GHMM_OK;
    ghmm_pd_region r{reads, n_reads, haps, n_haps};
    return ghmm_pd_compute_regions(ctx, &r, 1, out);
}


}  // extern "C"
