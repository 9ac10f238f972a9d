// runtime_internal.h -- what the host runtime's translation units share: the opaque structs behind the C-ABI
// handles (ghmm_ctx, ghmm_batch, ghmm_queue), the input views, and the functions that marshal, upload and run a
// batch (batch.cpp), pipeline and stream batches (queue.cpp), run PD-HMM batches (pd_host.cpp) and prepare raw
// reads (raw_host.cpp); runtime.cpp holds the context and the rest of the C-ABI.
#pragma once

#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <condition_variable>
#include <cstdint>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/ghmm.h"
#include "ghmm_internal.h"
#include "host_util.h"
#include "tables.h"

namespace ghmm {
namespace rt {

constexpr int kBlock = 128;
constexpr int kWarpsPerBlock = kBlock / 32;
// Default of ghmm_tuning.route_fp64_below: the FP32 pass can represent log10 L down to about -64 (the rerun
// threshold); a read expected 36 decades below that goes to FP64 without trying.
constexpr int kRouteFp64Log10 = -100;

struct Bucket {
    int key;  // rows-per-lane | 16 if multi-strip
    int begin, count;
    int grid;
};

// Routing of reads whose gap penalties are only known after the device imputation (DRAGstr).  The checks that
// guard against wrong finite results (a continuation penalty of 0, a matchToMatch probability of about 0) are
// decided for the whole batch from every value the imputation tables can produce.  The growth checks only save
// work: a pair whose rescaled FP32 or FP64 state overflows sums to a non-finite value and moves on to the next tier.
struct RouteBound {
    uint8_t force = 0;  // flags every read gets (bit0 FP64, bit2 exact FP64 tier)
};

// Input view shared by the region-array and flat entry points.
struct Source {
    // either regions (per-read pointers) ...
    const ghmm_region *regions = nullptr;
    int64_t n_regions = 0;
    // ... or flat planes
    const ghmm_flat *flat = nullptr;
    const RouteBound *bound = nullptr;  // set when the device rewrites the gap penalties after the upload
    // PD-HMM batches: per region 1 = no read-pair tasks (every pair to the general PD kernel)
    const uint8_t *region_direct = nullptr;
};

}  // namespace rt
}  // namespace ghmm

using namespace ghmm;
using namespace ghmm::rt;

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
    DevBuf<float2> d_read_scale;  // per read: the FP32 pass's log2 a_R as (2^-(la - n), n), from launch_read_scale
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
        d_scratch32.release(); d_scratch64.release(); d_read_scale.release(); d_post.release(); h_pd.release();
        d_pd.release();
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
    ghmm_batch pd_batch[2];    // the one-shot PD-HMM entry points' two pipeline slots, reused across calls
    cudaStream_t pd_stream2 = nullptr;  // the second slot's stream (created on first use)
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
    // each batch's kernels wait for the FP32 pass of the batch in the other slot (streaming queues, large pipelined calls)
    bool serial_fp32 = false;
    // worker-owned
    ghmm_batch slot[2];
    cudaStream_t stream[2]{};
    std::unique_ptr<QueueUnit> inflight[2];
    int64_t inflight_seq[2]{};
    int64_t seq = 0;
};

namespace ghmm {
namespace rt {

struct RawView {
    std::vector<ghmm_region> regions;
    std::unique_ptr<ghmm_read[]> reads;  // every region's reads, region after region (each entry written once, in
                                         // parallel: not zero-filled first)
    std::vector<uint8_t> q45, qgcp;  // shared constant planes
    std::vector<int32_t> mapq;
    int32_t max_len = 0;
    bool has_bound = false;
    RouteBound bound;
};

// runtime.cpp: status and message of a failed call (into the queue worker's own message on its thread)
extern thread_local std::string *t_error_sink;
int fail(ghmm_ctx *ctx, int code, const std::string &msg);
int cuda_fail(ghmm_ctx *ctx, cudaError_t e, const char *what);

// batch.cpp
int batch_marshal(ghmm_ctx *ctx, const Source &src, ghmm_batch &b);
uint8_t base_index(uint8_t b);  // column-code base index of a haplotype byte: A, C, G, T = 0..3, anything else 4
int batch_upload(ghmm_ctx *ctx, ghmm_batch &b, cudaStream_t s);
int fill_fp64_all(ghmm_ctx *ctx, ghmm_batch &b);
int batch_forward(ghmm_ctx *ctx, ghmm_batch &b, int mode);
int batch_enqueue(ghmm_ctx *ctx, ghmm_batch &b, int mode, cudaStream_t s);
int batch_finish(ghmm_ctx *ctx, ghmm_batch &b);
int batch_results(ghmm_ctx *ctx, ghmm_batch &b, double *out);
int batch_results_on(ghmm_ctx *ctx, ghmm_batch &b, double *out, cudaStream_t s);
int pd_forward_enqueue(ghmm_ctx *ctx, ghmm_batch &b, bool fp32, cudaStream_t s);
int pd_forward_finish(ghmm_ctx *ctx, ghmm_batch &b);

// queue.cpp.  Large synchronous inputs run as a pipeline of batches through the context's own queue: the first
// batch is small so that the GPU starts early, later ones grow to a third of the input.  Below 1.5e11 cells one batch
// is faster, the marshal being shorter than what the extra batches' launches and kernel tails cost (workload 1 end to
// end at 1,000 regions, 1.09e11 cells: 38.7 ms in one batch against 42.4 ms in three).
constexpr int64_t kPipelineMinCells = (int64_t)1.5e11;
int queue_open(ghmm_ctx *ctx, int64_t batch_cells, ghmm_queue **out, const ghmm_read_prep *raw_prep = nullptr,
               const RouteBound *bound = nullptr);
void queue_close(ghmm_queue *q);
int queue_status(ghmm_queue *q);
void queue_submit(ghmm_queue *q, std::unique_ptr<QueueUnit> u);
int queue_wait_all(ghmm_queue *q);
// Raw reads (mapq non-NULL, src.regions over the raw view's reads): every batch gets the read preparation prep on
// the device after its upload.
int pipelined_compute(ghmm_ctx *ctx, const Source &src, const std::vector<int64_t> &reg_cells,
                      const std::vector<int64_t> &reg_out, double *out, const int32_t *mapq = nullptr,
                      int32_t max_len = 0, const ghmm_read_prep *prep = nullptr, const RouteBound *bound = nullptr);
bool region_sizes(const Source &src, std::vector<int64_t> &cells, std::vector<int64_t> &outo, int threads);
int compute_sync(ghmm_ctx *ctx, const Source &src, double *out);
// cells from which a pipelined call takes the large schedule (growing chunks, FP32 passes in turn)
constexpr int64_t kPipelineLargeCells = (int64_t)5e11;
std::vector<int64_t> pipeline_cuts(const std::vector<int64_t> &cells);  // region cuts of a pipelined call

// pd_host.cpp
int pd_marshal(ghmm_ctx *ctx, const ghmm_pd_region *regs, int64_t G, ghmm_batch &b, const RouteBound *bound);
int pd_upload(ghmm_ctx *ctx, ghmm_batch &b, cudaStream_t s);
int batch_forward_pd(ghmm_ctx *ctx, ghmm_batch &b, bool fp32);

// raw_host.cpp
extern const char *const kRawErrors[];
int raw_region_problem(const ghmm_raw_region &rg, int32_t *max_len);
int raw_view(ghmm_ctx *ctx, const ghmm_raw_region *raw, int64_t G, const ghmm_read_prep *prep, RawView &v);
int raw_prepare_device(ghmm_ctx *ctx, ghmm_batch &b, const int32_t *mapq, int32_t max_len, const ghmm_read_prep *prep,
                       cudaStream_t s);

}  // namespace rt
}  // namespace ghmm

#define GHMM_CUDA(call, what)                         \
    do {                                              \
        cudaError_t e__ = (call);                     \
        if (e__ != cudaSuccess) return cuda_fail(ctx, e__, what); \
    } while (0)
