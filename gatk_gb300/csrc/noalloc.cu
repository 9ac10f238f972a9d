// noalloc.cu -- the PairHMM forward for callers that cannot allocate GPU memory.
//
// Some callers cannot call cudaMalloc: code that runs inside another framework's memory pool or a
// fixed device-memory budget, a process that has to keep its footprint fixed after start-up, or a
// caller that cannot take the implicit synchronisation an allocation brings.  ghmm_forward_pairs_noalloc
// serves them: it computes log10 likelihoods of explicit (read, haplotype) pairs whose bytes the caller
// already holds in device memory, writes them to a device array the caller provides, and allocates
// nothing.  The kernel is a variant of the FP64 wavefront kernel (kernels.cu): one pair per warp, four
// rows per lane, strips of 128 rows for longer reads.  Its strip-boundary scratch and its Phred lookup
// tables live in the file-scope static __device__ arrays below, which every GPU that loads the library
// holds until the process exits (12 MiB of scratch plus 134 KiB of tables).
//
// Set-up: the first call on a device, with that device current, resolves the scratch array's device
// address with cudaGetSymbolAddress, copies the tables into their arrays and waits for the copies to land
// (cudaDeviceSynchronize), so that a kernel launched afterwards on any stream, blocking or not, reads them.
// That first call should therefore come before any stream capture.  Later calls only launch the kernel on
// the caller's stream.  The caller's current device is restored before every return.
//
// Input bytes are checked on the device, as the other entry points check them on the host: a pair whose
// read has a base quality above 254, or an insertion, deletion or gap-continuation penalty above 127, gets
// NaN as its result (the caller reads its outputs back and treats NaN as an input error), and so does a pair
// whose haplotype is longer than GHMM_NOALLOC_MAX_HAP_LEN although max_hap_len promised otherwise.
//
// Every call shares the one scratch array, and the array keeps the last call's contents.  Nothing in it
// needs to start at zero (each warp writes a strip boundary before it reads it), but calls that overlap
// on the GPU (on different streams, or from different host threads) race on it and must be serialised by
// the caller.
#include <cuda_runtime.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>

#include "../../include/ghmm.h"
#include "ghmm_internal.h"
#include "tables.h"

namespace {

constexpr int kK = 4;          // rows per lane
constexpr int kS = 32 * kK;    // rows per strip
constexpr int kBlock = 128;
constexpr int kWarps = GHMM_NOALLOC_WARPS;
constexpr int kMaxCols = GHMM_NOALLOC_MAX_HAP_LEN;
constexpr unsigned kFull = 0xffffffffu;
constexpr double kLog10Scale64 = 307.0505955772608;  // log10(2^1020)

// strip-boundary rows (M, I, D of the last row of a strip, per haplotype column), one slice per warp
static __device__ __align__(256) double g_noalloc_scratch[(size_t)kWarps * kMaxCols * 3];
// Phred tables: 10^(-q/10), 1 - 10^(-q/10), 10^(-q/10)/3, matchToMatchProb(ins, del)
static __device__ __align__(256) double g_noalloc_err[256];
static __device__ __align__(256) double g_noalloc_prob[256];
static __device__ __align__(256) double g_noalloc_err3[256];
static __device__ __align__(256) double g_noalloc_m2m[128 * 128];

std::mutex g_setup_mu;
bool g_ready[256];
double *g_scratch_addr[256];

// messages are read back with ghmm_last_error(NULL, ...)
void set_error(const char *m) { ghmm::set_global_error(m); }

__global__ void __launch_bounds__(kBlock) noalloc_pairs_kernel(ghmm_dev_pairs in, double *out, double *scratch_base) {
    const int lane = threadIdx.x & 31;
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    double *scratch = scratch_base + warp * (int64_t)kMaxCols * 3;
    for (int64_t p = warp; p < in.n_pairs; p += nwarps) {
        const int read = in.pair_read[p], hap = in.pair_hap[p];
        const int64_t roff = in.read_off[read];
        const int R = (int)(in.read_off[read + 1] - roff);
        const int64_t hoff = in.hap_off[hap];
        const int H = (int)(in.hap_off[hap + 1] - hoff);
        if (H > kMaxCols) {  // beyond the scratch bound: flagged as NaN, never a silent value
            if (lane == 0) out[p] = __longlong_as_double(0x7ff8000000000000LL);
            continue;
        }
        if (R == 0 || H == 0) {
            if (lane == 0) out[p] = -INFINITY;
            continue;
        }
        // the read's bytes against the ranges the other entry points enforce (runtime.cpp): flagged as NaN
        bool bad = false;
        for (int i = lane; i < R; i += 32)
            bad |= in.quals[roff + i] > ghmm::kMaxQual || in.ins_gop[roff + i] > 127 || in.del_gop[roff + i] > 127 ||
                   in.gcp[roff + i] > 127;
        if (__any_sync(kFull, bad)) {
            if (lane == 0) out[p] = __longlong_as_double(0x7ff8000000000000LL);
            continue;
        }
        const double init = ldexp(1.0, 1020) / (double)H;
        const int nstrips = (R + kS - 1) / kS;
        const int pad = nstrips * kS - R;
        const uint8_t *hb = in.hap_bases + hoff;
        double acc = 0.0;
        for (int strip = 0; strip < nstrips; ++strip) {
            double pm[kK], pe[kK], tmm[kK], tim[kK], tmi[kK], tii[kK], tmd[kK], tdd[kK];
            uint32_t rbase[kK];
#pragma unroll
            for (int k = 0; k < kK; ++k) {
                const int pos = strip * kS + lane * kK + k - pad;
                if (pos < 0) {  // rows above the read reproduce the row-0 boundary
                    pm[k] = pe[k] = tmm[k] = tim[k] = tmi[k] = tii[k] = tmd[k] = 0.0;
                    tdd[k] = 1.0;
                    rbase[k] = 0x100u;
                } else {
                    const uint8_t base = in.bases[roff + pos], q = in.quals[roff + pos];
                    const uint8_t ins = in.ins_gop[roff + pos], del = in.del_gop[roff + pos];
                    const uint8_t gcp = in.gcp[roff + pos];
                    pm[k] = g_noalloc_prob[q];
                    pe[k] = base == 'N' ? pm[k] : g_noalloc_err3[q];
                    tmm[k] = g_noalloc_m2m[ins * 128 + del];  // all <= 127: checked above
                    tim[k] = g_noalloc_prob[gcp];
                    tmi[k] = g_noalloc_err[ins];
                    tii[k] = g_noalloc_err[gcp];
                    tmd[k] = g_noalloc_err[del];
                    tdd[k] = tii[k];
                    rbase[k] = base;
                }
            }
            double Mp[kK], Ip[kK], Dp[kK];
#pragma unroll
            for (int k = 0; k < kK; ++k) {
                Mp[k] = Ip[k] = 0.0;
                Dp[k] = ((strip == 0) && (lane * kK + k < pad)) ? init : 0.0;
            }
            double gM = 0.0, gI = 0.0;
            double gD = ((strip == 0) && (lane * kK - 1 < pad)) ? init : 0.0;
            const bool last_strip = strip == nstrips - 1;
            double nxM = 0.0, nxI = 0.0, nxD = 0.0;
            if (strip > 0 && lane == 0) {
                nxM = scratch[0];
                nxI = scratch[1];
                nxD = scratch[2];
            }
            for (int s = 0; s < H + 31; ++s) {
                const int c = s - lane;
                const bool valid = c >= 0 && c < H;
                const uint32_t y = valid ? (uint32_t)hb[c] : 0x200u;
                const bool yn = (y == 'N');
                double uM = __shfl_up_sync(kFull, Mp[kK - 1], 1);
                double uI = __shfl_up_sync(kFull, Ip[kK - 1], 1);
                double uD = __shfl_up_sync(kFull, Dp[kK - 1], 1);
                if (c == 0) {  // column-0 boundary (lanes compute ahead of their first column)
#pragma unroll
                    for (int k = 0; k < kK; ++k) {
                        Mp[k] = Ip[k] = 0.0;
                        Dp[k] = ((strip == 0) && (lane * kK + k < pad)) ? init : 0.0;
                    }
                    gM = gI = 0.0;
                    gD = ((strip == 0) && (lane * kK - 1 < pad)) ? init : 0.0;
                }
                if (lane == 0) {
                    if (strip == 0) {
                        uM = 0.0;
                        uI = 0.0;
                        uD = init;
                    } else {
                        uM = nxM;
                        uI = nxI;
                        uD = nxD;
                        if (c + 1 < H) {
                            nxM = scratch[3 * (c + 1) + 0];
                            nxI = scratch[3 * (c + 1) + 1];
                            nxD = scratch[3 * (c + 1) + 2];
                        }
                    }
                }
#pragma unroll
                for (int k = kK - 1; k >= 0; --k) {
                    const double dM = k ? Mp[k - 1] : gM;
                    const double dI = k ? Ip[k - 1] : gI;
                    const double dD = k ? Dp[k - 1] : gD;
                    const double prior = (rbase[k] == y || yn) ? pm[k] : pe[k];
                    const double Mn = prior * fma(dM, tmm[k], (dI + dD) * tim[k]);
                    const double Dn = fma(Dp[k], tdd[k], Mp[k] * tmd[k]);
                    Mp[k] = Mn;
                    Dp[k] = Dn;
                }
                double aM = uM, aI = uI;
#pragma unroll
                for (int k = 0; k < kK; ++k) {
                    const double In = fma(aI, tii[k], aM * tmi[k]);
                    Ip[k] = In;
                    aM = Mp[k];
                    aI = In;
                }
                gM = uM;
                gI = uI;
                gD = uD;
                if (valid && lane == 31) {
                    if (last_strip) {
                        acc += Mp[kK - 1] + Ip[kK - 1];
                    } else {
                        scratch[3 * c + 0] = Mp[kK - 1];
                        scratch[3 * c + 1] = Ip[kK - 1];
                        scratch[3 * c + 2] = Dp[kK - 1];
                    }
                }
            }
            __syncwarp();
        }
        if (lane == 31) out[p] = log10(acc) - kLog10Scale64;
    }
}

// Once per device, with that device current: resolve the scratch address and fill the tables.
int setup_device(int device) {
    std::lock_guard<std::mutex> lk(g_setup_mu);
    if (g_ready[device]) return GHMM_OK;
    void *addr = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess || addr == nullptr) {
        set_error("cudaGetSymbolAddress of the no-allocation scratch array failed");
        return GHMM_ERR_CUDA;
    }
    static ghmm::HostTables t;  // static storage: built once
    ghmm::build_host_tables(t);
    if (cudaMemcpyToSymbol(g_noalloc_err, t.err, sizeof t.err) != cudaSuccess ||
        cudaMemcpyToSymbol(g_noalloc_prob, t.prob, sizeof t.prob) != cudaSuccess ||
        cudaMemcpyToSymbol(g_noalloc_err3, t.err3, sizeof t.err3) != cudaSuccess ||
        cudaMemcpyToSymbol(g_noalloc_m2m, t.m2m, sizeof t.m2m) != cudaSuccess) {
        set_error("copying the Phred tables into the no-allocation arrays failed");
        return GHMM_ERR_CUDA;
    }
    // the copies above come from pageable memory and may return before their DMA lands; wait for them once, so
    // that the first kernel reads the tables whatever stream it is launched on
    e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
        set_error("waiting for the no-allocation tables to land failed");
        return GHMM_ERR_CUDA;
    }
    g_scratch_addr[device] = (double *)addr;
    g_ready[device] = true;
    return GHMM_OK;
}

}  // namespace

extern "C" int ghmm_forward_pairs_noalloc(int32_t device, const ghmm_dev_pairs *in, double *d_out, void *stream) {
    if (!in || !d_out) {
        set_error("ghmm_forward_pairs_noalloc: NULL argument");
        return GHMM_ERR_ARG;
    }
    if (in->max_hap_len < 0 || in->max_hap_len > GHMM_NOALLOC_MAX_HAP_LEN) {
        set_error("ghmm_forward_pairs_noalloc: haplotypes longer than GHMM_NOALLOC_MAX_HAP_LEN (2048) are not "
                  "supported by the no-allocation entry point; use ghmm_batch_* instead");
        return GHMM_ERR_ARG;
    }
    if (in->n_pairs < 0 || in->n_pairs > (int64_t)INT32_MAX) {
        set_error("ghmm_forward_pairs_noalloc: pair count out of range");
        return GHMM_ERR_ARG;
    }
    if (device < 0 || device >= 256) {
        set_error("ghmm_forward_pairs_noalloc: device ordinal out of range");
        return GHMM_ERR_ARG;
    }
    if (in->n_pairs == 0) return GHMM_OK;
    if (!in->bases || !in->quals || !in->ins_gop || !in->del_gop || !in->gcp || !in->read_off || !in->hap_bases ||
        !in->hap_off || !in->pair_read || !in->pair_hap) {
        set_error("ghmm_forward_pairs_noalloc: NULL device array");
        return GHMM_ERR_ARG;
    }
    int cur = -1;
    if (cudaGetDevice(&cur) != cudaSuccess) {
        set_error("ghmm_forward_pairs_noalloc: cudaGetDevice failed");
        return GHMM_ERR_CUDA;
    }
    if (cur != device && cudaSetDevice(device) != cudaSuccess) {
        set_error("ghmm_forward_pairs_noalloc: cudaSetDevice failed");
        cudaSetDevice(cur);
        return GHMM_ERR_CUDA;
    }
    int rc = setup_device(device);
    if (rc == GHMM_OK) {
        const int64_t want_blocks = (in->n_pairs + (kBlock / 32) - 1) / (kBlock / 32);
        const int grid = (int)(want_blocks < kWarps / (kBlock / 32) ? want_blocks : kWarps / (kBlock / 32));
        noalloc_pairs_kernel<<<grid, kBlock, 0, (cudaStream_t)stream>>>(*in, d_out, g_scratch_addr[device]);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error(cudaGetErrorString(e));
            rc = GHMM_ERR_CUDA;
        }
    }
    if (cur != device) cudaSetDevice(cur);  // the caller's current device, as it was
    return rc;
}
