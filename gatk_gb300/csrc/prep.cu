// prep.cu -- read preparation before the PairHMM, on the device: what PairHMMLikelihoodCalculationEngine.
// modifyReadQualities does to each read on the host in GATK (src/main/java/org/broadinstitute/hellbender/tools/
// walkers/haplotypecaller/PairHMMLikelihoodCalculationEngine.java:283-322,331-371):
//   - the PCR indel error model: at every position but the last, insertion and deletion qualities are capped by the
//     model's quality for the tandem-repeat length there (findTandemRepeatUnits, ReadLikelihoodCalculationEngine.
//     java:193-253, repeat units up to 8 bases, lengths capped at 20);
//   - base qualities capped by the mapping quality (unless disabled), then base qualities below the threshold and
//     insertion / deletion qualities below 6 set to 6 (compared as Java's signed bytes).
// The batch's planes hold the raw values (missing insertion / deletion qualities as 45, the constant gap continuation
// penalty filled in); this kernel rewrites quals, ins and dels in place, one thread per read.
#include <cuda_runtime.h>

#include <cstdint>

#include "ghmm_internal.h"

namespace ghmm {
namespace {

constexpr int kMaxUnit = 8;
constexpr int kMaxRepeat = 20;

// findNumberOfRepetitions over sub-ranges of the read: copies of unit b[u, u+L) at the start (leading) or the end
// (trailing) of b[t, t+n)
__device__ int repetitions(const uint8_t *b, int u, int L, int t, int n, bool leading) {
    if (n == 0) return 0;
    int count = 0;
    if (leading) {
        for (int s = 0; s <= n - L; s += L) {
            for (int k = 0; k < L; ++k)
                if (b[t + s + k] != b[u + k]) return count;
            ++count;
        }
    } else {
        for (int s = n - L; s >= 0; s -= L) {
            for (int k = 0; k < L; ++k)
                if (b[t + s + k] != b[u + k]) return count;
            ++count;
        }
    }
    return count;
}

__device__ bool same_unit(const uint8_t *b, int u1, int l1, int u2, int l2) {
    if (l1 != l2) return false;
    for (int k = 0; k < l1; ++k)
        if (b[u1 + k] != b[u2 + k]) return false;
    return true;
}

// findTandemRepeatUnits(...).getRight() at `offset` of a read of n bases
__device__ int tandem_repeat_length(const uint8_t *b, int n, int offset) {
    int max_bw = 0, bw_u = offset, bw_l = 1;
    for (int L = 1; L <= kMaxUnit; ++L) {
        if (offset + 1 - L < 0) break;
        max_bw = repetitions(b, offset - L + 1, L, 0, offset + 1, false);
        if (max_bw > 1) {
            bw_u = offset - L + 1;
            bw_l = L;
            break;
        }
    }
    int max_rl = max_bw;
    if (offset < n - 1) {
        int fw_u = offset + 1, fw_l = 1, max_fw = 0;
        for (int L = 1; L <= kMaxUnit; ++L) {
            if (offset + L + 1 > n) break;
            max_fw = repetitions(b, offset + 1, L, offset + 1, n - offset - 1, true);
            if (max_fw > 1) {
                fw_l = L;
                break;
            }
        }
        if (same_unit(b, fw_u, fw_l, bw_u, bw_l))
            max_rl = max_bw + max_fw;
        else
            max_rl = max_fw + repetitions(b, fw_u, fw_l, 0, offset + 1, false);
    }
    return max_rl > kMaxRepeat ? kMaxRepeat : max_rl;
}

__device__ __forceinline__ int as_java_byte(int v) { return v > 127 ? v - 256 : v; }

__global__ void prep_kernel(DevBatch B, uint8_t *quals, uint8_t *ins, uint8_t *dels, int64_t n_reads, PrepArgs P) {
    for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < n_reads; r += (int64_t)gridDim.x * blockDim.x) {
        const int64_t o = B.read_off[r];
        const int n = (int)(B.read_off[r + 1] - o);
        const uint8_t *b = B.bases + o;
        if (P.pcr) {
            for (int i = 1; i < n; ++i) {
                const int cap = P.pcr_cache[tandem_repeat_length(b, n, i - 1)];
                if (ins[o + i - 1] > cap) ins[o + i - 1] = (uint8_t)cap;
                if (dels[o + i - 1] > cap) dels[o + i - 1] = (uint8_t)cap;
            }
        }
        const int mapq = P.mapq[r];
        for (int i = 0; i < n; ++i) {
            int q = quals[o + i];
            if (P.cap_to_mapq) q = (q < mapq ? q : mapq) & 0xFF;
            if (as_java_byte(q) < P.threshold) q = 6;
            quals[o + i] = (uint8_t)q;
            if (as_java_byte(ins[o + i]) < 6) ins[o + i] = 6;
            if (as_java_byte(dels[o + i]) < 6) dels[o + i] = 6;
        }
    }
}

}  // namespace

int launch_prep(const DevBatch &b, int64_t n_reads, const PrepArgs &p, int sm_count, cudaStream_t s) {
    if (n_reads <= 0) return 0;
    const int block = 128;
    const int64_t want = (n_reads + block - 1) / block;
    const int grid = (int)(want < (int64_t)sm_count * 8 ? want : (int64_t)sm_count * 8);
    // the planes are the batch's own device buffers (DevBatch holds them as const for the forward kernels)
    prep_kernel<<<grid, block, 0, s>>>(b, const_cast<uint8_t *>(b.quals), const_cast<uint8_t *>(b.ins),
                                       const_cast<uint8_t *>(b.dels), n_reads, p);
    return (int)cudaGetLastError();
}

}  // namespace ghmm
