// host_util.h -- host-side helpers shared by the runtime (runtime.cpp) and the Smith-Waterman host code
// (sw_host.cpp): device and pinned buffers that grow, a thread pool loop, and the context and batch views the
// Smith-Waterman code needs from the runtime.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstdint>
#include <string>
#include <thread>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "ghmm_internal.h"

struct ghmm_ctx;
struct ghmm_batch;

namespace ghmm {

// An NVTX range over a host phase (marshalling, upload, launches, planning), visible to Nsight tools; without a
// tool attached the calls return at once
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Test hook (ghmm_debug_inject): the number of device allocations still to be refused as out of memory
extern std::atomic<int64_t> g_refuse_allocations;

template <typename T>
struct DevBuf {
    T *p = nullptr;
    size_t cap = 0;
    cudaError_t reserve(size_t n) {
        if (n <= cap && p) return cudaSuccess;
        if (g_refuse_allocations.load(std::memory_order_relaxed) > 0 && g_refuse_allocations.fetch_sub(1) > 0)
            return cudaErrorMemoryAllocation;
        // a buffer that has to grow again grows by a quarter more than asked, so that batches of slowly
        // rising size do not free (and so synchronise the device) every time
        const size_t want = std::max<size_t>(cap ? std::max(n, cap + cap / 4) : n, 1);
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
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
        const size_t want = std::max<size_t>(cap ? std::max(n, cap + cap / 4) : n, 1);
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
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

inline int hw_threads(int requested) {
    const int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    return requested > 0 ? std::min(requested, hw) : hw;
}

// f(i) for i in [0, n) on up to `threads` threads, the calling thread one of them.  Threads take `grain`
// consecutive indices at a time; grain 0 (the default) takes about a quarter of an even share, at most 64, so
// that a loop over a few dozen regions or blocks still spreads over all threads.
template <typename F>
inline void parallel_for(int64_t n, int threads, F f, int64_t grain = 0) {
    if (n <= 0) return;
    threads = std::max(threads, 1);
    if (grain <= 0) grain = std::min<int64_t>(64, std::max<int64_t>(1, n / ((int64_t)threads * 4)));
    threads = (int)std::min<int64_t>(threads, (n + grain - 1) / grain);
    if (threads <= 1) {
        for (int64_t i = 0; i < n; i++) f(i);
        return;
    }
    std::atomic<int64_t> next{0};
    auto work = [&] {
        for (;;) {
            const int64_t i0 = next.fetch_add(grain);
            if (i0 >= n) break;
            const int64_t i1 = std::min(n, i0 + grain);
            for (int64_t i = i0; i < i1; i++) f(i);
        }
    };
    std::vector<std::thread> pool;
    pool.reserve((size_t)threads - 1);
    for (int t = 1; t < threads; t++) pool.emplace_back(work);
    work();
    for (auto &th : pool) th.join();
}

struct SwEngine;
void sw_engine_destroy(SwEngine *e);

// What the Smith-Waterman entry points need from a context (runtime.cpp).
struct CtxInfo {
    int device = 0, sm_count = 0, threads = 0;
    cudaStream_t stream = nullptr;
    SwEngine **sw = nullptr;  // the context's Smith-Waterman buffers, created on first use
};
// GHMM_ERR_STATE when the context is NULL or closed.
int ctx_info(ghmm_ctx *ctx, CtxInfo *info);
// Records msg as the context's last error and returns code.
int ctx_fail(ghmm_ctx *ctx, int code, const std::string &msg);

// A batch's device view and host offsets (runtime.cpp): read_off[n_reads + 1], hap_off[n_haps + 1],
// region_read_off[n_regions + 1], region_hap_off[n_regions + 1], out_off[n_regions + 1], back to back.
struct BatchInfo {
    const DevBatch *dev = nullptr;
    const int64_t *h_off = nullptr;
    int64_t n_regions = 0, n_reads = 0, n_haps = 0;
    bool has_results = false;  // uploaded and run at least once
};
void batch_info(const ghmm_batch *b, BatchInfo *info);

}  // namespace ghmm
