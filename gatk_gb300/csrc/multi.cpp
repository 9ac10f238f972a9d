// multi.cpp -- one caller driving several GPUs (include/ghmm.h, "Several devices").
//
// HaplotypeCaller's JVM is one process; its host-side parallelism today is GKL's thread count
// (HC/PairHMMNativeArgumentCollection.java:11-12) or one likelihood engine per Spark partition
// (tools/HaplotypeCallerSpark.java:175-179).  Here one handle owns one context (stream, buffers, tables) per
// device and splits each call's work between them.  Pairs are independent, so the split needs no
// device-to-device traffic and no collective: the caller's reads, numbered in region order, are cut into
// one contiguous range per device so that every range carries about the same number of cells
// (sum over its reads of read length x the summed lengths of its region's haplotypes).  Because results are
// read-major per region and regions follow each other, a contiguous range of reads owns a contiguous slice of
// the caller's `out`, and each device's results land straight in that slice.  A range may start or end in
// the middle of a region: that device sees the region with a subset of its reads and all its haplotypes.
//
// The devices run on one host thread each; every context marshals with its share of the host cores.
// Layered on the single-device C-ABI (ghmm_initialize / ghmm_compute_regions / ghmm_done).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ghmm.h"

struct ghmm_multi {
    std::vector<int32_t> devices;
    std::vector<ghmm_ctx *> ctx;  // empty when the devices are stubs (GHMM_MULTI_STUB_DEVICES)
    bool stub = false;
    std::string last_error;
};

namespace {

// Cells of every read (its length times its region's summed haplotype length), reads numbered in region order.
// Returns false on a malformed region array.
bool read_costs(const ghmm_region *regions, int32_t n_regions, std::vector<int64_t> &cost,
                std::vector<int64_t> &out_per_read, std::string &err) {
    cost.clear();
    out_per_read.clear();
    for (int32_t g = 0; g < n_regions; g++) {
        const ghmm_region &rg = regions[g];
        if (rg.n_reads < 0 || rg.n_haps < 0 || (rg.n_reads > 0 && !rg.reads) || (rg.n_haps > 0 && !rg.haps)) {
            err = "region " + std::to_string(g) + ": negative count or NULL array";
            return false;
        }
        int64_t hap_cols = 0;
        for (int32_t h = 0; h < rg.n_haps; h++) hap_cols += std::max<int32_t>(rg.haps[h].length, 0);
        for (int32_t r = 0; r < rg.n_reads; r++) {
            cost.push_back((int64_t)std::max<int32_t>(rg.reads[r].length, 0) * hap_cols);
            out_per_read.push_back(rg.n_haps);
        }
    }
    return true;
}

// Contiguous split of the reads into n ranges of about equal cells: range d ends at the first read boundary where
// the running total reaches (d + 1) / n of the whole (or the nearer of the two boundaries around that point).
void plan(const std::vector<int64_t> &cost, const std::vector<int64_t> &out_per_read, int32_t n,
          ghmm_multi_slice *slices) {
    const int64_t nr = (int64_t)cost.size();
    int64_t total = 0;
    for (int64_t c : cost) total += c;
    int64_t r = 0, run = 0, out = 0;
    for (int32_t d = 0; d < n; d++) {
        ghmm_multi_slice &s = slices[d];
        s.read_begin = r;
        s.out_begin = out;
        s.cells = 0;
        const long double target = (long double)total * (d + 1) / n;
        if (d == n - 1) {
            for (; r < nr; r++) {
                run += cost[(size_t)r];
                s.cells += cost[(size_t)r];
                out += out_per_read[(size_t)r];
            }
        } else {
            while (r < nr && (long double)run + cost[(size_t)r] <= target) {
                run += cost[(size_t)r];
                s.cells += cost[(size_t)r];
                out += out_per_read[(size_t)r];
                r++;
            }
            // take the straddling read too when that lands closer to the target
            if (r < nr && (long double)run + cost[(size_t)r] - target < target - (long double)run) {
                run += cost[(size_t)r];
                s.cells += cost[(size_t)r];
                out += out_per_read[(size_t)r];
                r++;
            }
        }
        s.read_end = r;
        s.out_end = out;
    }
}

// The regions of a read range: every region that overlaps it, restricted to the overlapping reads.
std::vector<ghmm_region> sub_regions(const ghmm_region *regions, int32_t n_regions, int64_t read_begin,
                                     int64_t read_end) {
    std::vector<ghmm_region> sub;
    int64_t first = 0;
    for (int32_t g = 0; g < n_regions && first < read_end; g++) {
        const ghmm_region &rg = regions[g];
        const int64_t a = std::max<int64_t>(read_begin, first), b = std::min<int64_t>(read_end, first + rg.n_reads);
        if (a < b) sub.push_back(ghmm_region{rg.reads + (a - first), (int32_t)(b - a), rg.haps, rg.n_haps});
        first += rg.n_reads;
    }
    return sub;
}

int fail(ghmm_multi *m, int code, const std::string &msg) {
    if (m) m->last_error = msg;
    return code;
}

}  // namespace

extern "C" {

int ghmm_multi_plan(const ghmm_region *regions, int32_t n_regions, int32_t n_devices, ghmm_multi_slice *slices) {
    if (n_devices < 1 || !slices || n_regions < 0 || (n_regions > 0 && !regions)) return GHMM_ERR_ARG;
    std::vector<int64_t> cost, outs;
    std::string err;
    if (!read_costs(regions, n_regions, cost, outs, err)) return GHMM_ERR_ARG;
    plan(cost, outs, n_devices, slices);
    return GHMM_OK;
}

int ghmm_multi_create(const int32_t *devices, int32_t n_devices, const ghmm_args *args, ghmm_multi **out) {
    if (!out) return GHMM_ERR_ARG;
    *out = nullptr;
    if (n_devices < 1 || !devices) return GHMM_ERR_ARG;
    auto *m = new ghmm_multi();
    m->devices.assign(devices, devices + n_devices);
    const char *stub = getenv("GHMM_MULTI_STUB_DEVICES");
    m->stub = stub && stub[0] && strcmp(stub, "0") != 0;
    if (!m->stub) {
        ghmm_args a{0, 0, 0, 0};
        if (args) a = *args;
        if (a.max_threads <= 0) {  // the host cores, shared between the devices' marshalling
            const unsigned hc = std::max(1u, std::thread::hardware_concurrency());
            a.max_threads = (int32_t)std::max<unsigned>(1, hc / (unsigned)n_devices);
        }
        for (int32_t d = 0; d < n_devices; d++) {
            a.device = devices[d];
            ghmm_ctx *c = nullptr;
            const int rc = ghmm_initialize(&a, &c);
            if (rc != GHMM_OK) {
                for (ghmm_ctx *x : m->ctx) ghmm_done(x);
                delete m;
                return rc;  // the message stays readable through ghmm_last_error(NULL, ...)
            }
            m->ctx.push_back(c);
        }
    }
    *out = m;
    return GHMM_OK;
}

int ghmm_multi_compute_regions(ghmm_multi *m, const ghmm_region *regions, int32_t n_regions, double *out) {
    if (!m) return GHMM_ERR_STATE;
    if (n_regions < 0 || (n_regions > 0 && !regions)) return fail(m, GHMM_ERR_ARG, "bad region array");
    std::vector<int64_t> cost, outs;
    std::string err;
    if (!read_costs(regions, n_regions, cost, outs, err)) return fail(m, GHMM_ERR_ARG, err);
    const int32_t n = (int32_t)m->devices.size();
    std::vector<ghmm_multi_slice> slices((size_t)n);
    plan(cost, outs, n, slices.data());
    if (slices.back().out_end > 0 && !out) return fail(m, GHMM_ERR_ARG, "NULL output");
    std::vector<int> rc((size_t)n, GHMM_OK);
    std::vector<std::string> msg((size_t)n);
    auto run = [&](int32_t d) {
        const ghmm_multi_slice &s = slices[(size_t)d];
        if (s.read_begin == s.read_end) return;
        std::vector<ghmm_region> sub = sub_regions(regions, n_regions, s.read_begin, s.read_end);
        if (m->stub) {  // host-only stand-in: subtract (device + 1) over the slice the sub-regions' outputs fill
            int64_t k = 0;
            for (const ghmm_region &rg : sub) k += (int64_t)rg.n_reads * rg.n_haps;
            if (k != s.out_end - s.out_begin) {
                rc[(size_t)d] = GHMM_ERR_STATE;
                msg[(size_t)d] = "stub device: sub-region outputs do not fill the slice";
                return;
            }
            for (int64_t i = s.out_begin; i < s.out_end; i++) out[i] -= (double)(d + 1);
            return;
        }
        rc[(size_t)d] = ghmm_compute_regions(m->ctx[(size_t)d], sub.data(), (int32_t)sub.size(), out + s.out_begin);
        if (rc[(size_t)d] != GHMM_OK) {
            char buf[1024];
            ghmm_last_error(m->ctx[(size_t)d], buf, sizeof buf);
            msg[(size_t)d] = buf;
        }
    };
    std::vector<std::thread> th;
    for (int32_t d = 1; d < n; d++) th.emplace_back(run, d);
    run(0);
    for (auto &t : th) t.join();
    for (int32_t d = 0; d < n; d++)
        if (rc[(size_t)d] != GHMM_OK)
            return fail(m, rc[(size_t)d], "device " + std::to_string(m->devices[(size_t)d]) + ": " + msg[(size_t)d]);
    return GHMM_OK;
}

int ghmm_multi_context(ghmm_multi *m, int32_t index, ghmm_ctx **ctx) {
    if (!m || !ctx) return GHMM_ERR_ARG;
    if (index < 0 || index >= (int32_t)m->ctx.size()) return fail(m, GHMM_ERR_ARG, "no context at that index");
    *ctx = m->ctx[(size_t)index];
    return GHMM_OK;
}

int ghmm_multi_last_error(const ghmm_multi *m, char *buf, size_t n) {
    if (!m || !buf || n == 0) return GHMM_ERR_ARG;
    snprintf(buf, n, "%s", m->last_error.c_str());
    return GHMM_OK;
}

int ghmm_multi_destroy(ghmm_multi *m) {
    if (!m) return GHMM_OK;
    int rc = GHMM_OK;
    for (ghmm_ctx *c : m->ctx) {
        const int r = ghmm_done(c);
        if (r != GHMM_OK && rc == GHMM_OK) rc = r;
    }
    delete m;
    return rc;
}

}  // extern "C"
