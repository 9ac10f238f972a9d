// batch.cpp -- one batch of regions through the GPU: marshal (multi-threaded copy of every read's five byte arrays
// and every haplotype into pinned planes, haplotype column codes, validation and FP64 routing) -> build warp tasks
// (reads paired within a region by rows-per-lane bucket, longest first) -> async H2D -> the forward as two captured
// CUDA graphs (FP32 buckets and epilogue; the FP64 tiers) -> D2H -> validation of results (log10 L <= 0, not NaN;
// PairHMM.java:305-306).
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


// -------------------------------------------------------------------------------------------------
// Marshal inputs into the batch's pinned staging and build tasks.
int batch_marshal(ghmm_ctx *ctx, const Source &src, ghmm_batch &b) {
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
        struct ReadPair {
            int key;
            int64_t a, b;  // b < 0: a single read
        };
        std::vector<ReadPair> pairs;
        std::vector<std::pair<int, int64_t>> leftovers;  // (key, read) of the single-strip classes' odd reads
        std::vector<std::pair<int64_t, int64_t>> chunks;  // haplotype ranges of one task
        for (int64_t g = G * part / n_parts; g < G * (part + 1) / n_parts; g++) {
            const int64_t h0 = rho[(size_t)g], h1 = rho[(size_t)g + 1];
            const int64_t r0 = rro[(size_t)g], r1 = rro[(size_t)g + 1];
            if (h1 == h0 || r1 == r0) continue;
            bool region_fp64 = src.region_direct && src.region_direct[g];
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
            // neighbours of one class share a task; the single-strip classes' leftovers (one read of each class with
            // an odd count) then pair up with each other from the largest K down, each pair at the larger K (the
            // shorter read gets more dummy rows above it), so a region keeps at most one half-empty task
            pairs.clear();
            leftovers.clear();
            for (size_t i = 0; i < groups.size();) {
                const int64_t cls = groups[i].first / 100000;
                const int key = (int)(cls / 4096);
                const int64_t ra = groups[i].second;
                int64_t rb = -1;
                if (i + 1 < groups.size() && groups[i + 1].first / 100000 == cls) rb = groups[i + 1].second;
                i += (rb >= 0) ? 2 : 1;
                if (rb < 0 && !(key & 16))
                    leftovers.emplace_back(key, ra);
                else
                    pairs.push_back(ReadPair{key, ra, rb});
            }
            for (size_t i = leftovers.size(); i > 0;) {  // ascending keys: pair from the top
                if (i >= 2) {
                    pairs.push_back(ReadPair{leftovers[i - 1].first, leftovers[i - 1].second, leftovers[i - 2].second});
                    i -= 2;
                } else {
                    pairs.push_back(ReadPair{leftovers[0].first, leftovers[0].second, -1});
                    i -= 1;
                }
            }
            for (const ReadPair &rp : pairs) {
                const int key = rp.key;
                const int64_t ra = rp.a, rb = rp.b;
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
int batch_upload(ghmm_ctx *ctx, ghmm_batch &b, cudaStream_t s) {
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
    GHMM_CUDA(b.d_read_scale.reserve((size_t)std::max<int64_t>(NR, 1)), "device read scales");

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
    d.read_scale = b.d_read_scale.p;
    // the FP32 pass's per-read scale from the uploaded planes (raw batches redo it after their preparation)
    const int e = launch_read_scale(ctx->tables, d, NR, b.d_read_scale.p, ctx->sm_count, s);
    if (e) return cuda_fail(ctx, (cudaError_t)e, "read scale launch");
    b.uploaded = true;
    return GHMM_OK;
}

// FP64 mode: every (read, hap) pair of every region, read-major; reads marked exact-only go to the exact tier.
int fill_fp64_all(ghmm_ctx *ctx, ghmm_batch &b) {
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



int batch_forward(ghmm_ctx *ctx, ghmm_batch &b, int mode) {
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
int batch_phase(ghmm_ctx *ctx, ghmm_batch &b, int phase, cudaStream_t s) {
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

int capture_phase(ghmm_ctx *ctx, ghmm_batch &b, int phase, cudaStream_t s, cudaGraphExec_t *out) {
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

int kernel_launch_count(const ghmm_batch &b, int mode) {
    int n = 1;
    if (mode == GHMM_MODE_FP32_RERUN) n += (int)b.buckets.size() + (b.n_tasks > 0 ? 1 : 0);
    return n;
}

// Enqueue a forward on stream s without waiting: control words, FP64 pre-queue, the kernel graph, and the
// D2H of the counters.  batch_finish waits and reads the outcome.
int batch_enqueue(ghmm_ctx *ctx, ghmm_batch &b, int mode, cudaStream_t s) {
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

int batch_finish(ghmm_ctx *ctx, ghmm_batch &b) {
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

int batch_results(ghmm_ctx *ctx, ghmm_batch &b, double *out) { return batch_results_on(ctx, b, out, ctx->stream); }

// The results through pinned staging (a copy into the caller's pageable memory ran at about 1 GB/s), then copied out
// and checked (PairHMM.java:305-306) in parallel blocks.
int batch_results_on(ghmm_ctx *ctx, ghmm_batch &b, double *out, cudaStream_t s) {
    if (b.n_out == 0) return GHMM_OK;
    if (!out) return fail(ctx, GHMM_ERR_ARG, "NULL output");
    const int64_t n = b.n_out;
    GHMM_CUDA(b.h_out.reserve((size_t)n), "pinned results");
    GHMM_CUDA(cudaMemcpyAsync(b.h_out.p, b.d_out.p, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s), "D2H results");
    b.results_d2h = n * 8;
    GHMM_CUDA(cudaStreamSynchronize(s), "D2H results");
    const double *src = b.h_out.p;
    std::atomic<int64_t> bad{-1};
    parallel_for((n + (1 << 20) - 1) >> 20, hw_threads(ctx->max_threads), [&](int64_t k) {
        const int64_t a = k << 20, e = std::min<int64_t>(n, a + (1 << 20));
        for (int64_t i = a; i < e; i++) {
            const double v = src[i];
            out[i] = v;
            if (!(v <= 0.0)) {
                int64_t expect = -1;
                bad.compare_exchange_strong(expect, i);
            }
        }
    }, 1);
    if (bad.load() >= 0) {
        char msg[160];
        snprintf(msg, sizeof msg, "PairHMM log10 likelihood %g at output %lld is not a valid log10 probability",
                 src[bad.load()], (long long)bad.load());
        return fail(ctx, GHMM_ERR_RESULT, msg);
    }
    return GHMM_OK;
}



}  // namespace rt
}  // namespace ghmm
