// calib.cu -- differentiable PairHMM for gap-penalty calibration: forward log10 likelihoods and a
// hand-written backward (adjoint) pass with checkpointed forward recomputation.
//
// Model.  The LoglessPairHMM recurrence (src/main/java/org/broadinstitute/hellbender/utils/pairhmm/
// LoglessPairHMM.java:47-67) with continuous per-position gap parameters instead of Phred bytes.  For read
// position p (matrix row i = p + 1), g = gap-open log10-probability and c = gap-continuation log10-probability:
//     MI = MD = 10^g,   MM = 1 - 2*10^g,   II = DD = 10^c,   IM = 1 - 10^c
// (the form PairHMMModel.qualToTransProbs takes for equal insertion/deletion penalties, PairHMMModel.java:107-117,
// with the Jacobian-table matchToMatch replaced by its exact value).  Priors come from base qualities as in
// LoglessPairHMM.initializePriors (:79-93).  This is the parameter space of the DRAGstr model, whose per-(period,
// repeat) GOP/GCP tables (DragstrParams.java:49-117) set g and c of each read position.
//
// Kernel.  One warp per (read, haplotype) pair, K rows per lane (reads up to 256 bases in one strip of 32 K rows;
// longer reads in strips of 256 rows, K = 8), the anti-diagonal wavefront of the forward kernels: lane l computes
// column s - l at step s.  A strip's last row (M, I, D per column) is kept in scratch as the next strip's row above;
// the backward runs the strips last to first, and the adjoint values a strip's first row hands the row above are
// kept in scratch per column for the strip above it.
//  * Forward: the whole warp front (each lane's K rows of M, I, D plus the diagonal inputs) is saved to scratch
//    every kSeg steps (the checkpoints); lane 31 sums the last row into L_s (scaled likelihood).
//  * Backward: segments are processed last to first.  Each segment's forward is recomputed from its checkpoint,
//    keeping every step's front, and then the adjoint wavefront runs over it in reverse: lane l at reverse step s
//    handles column s - l, receiving from lane l+1 (the row below) by __shfl_down_sync.  Adjoints are seeded with
//    w / L_s at the last row, so beta * forward products are O(1) in FP32 (they sum to w * d ln L / d(.)).
//    Per row the six transition sensitivities are summed over columns and turned into
//        d(w log10 L)/dg = 10^g (G_MI + G_MD - 2 G_MM),   d(w log10 L)/dc = 10^c (G_II + G_DD - G_IM),
//    added atomically into per-read-position gradient arrays.
// T = float runs scale 2^120; a pair whose FP32 L_s falls below 1e-28 is redone with T = double (scale 2^1020).
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cstdint>

#include "../../include/ghmm.h"
#include "../../include/ghmm_calib.h"
#include "ghmm_internal.h"

namespace ghmm {
namespace {

constexpr unsigned kFullMask = 0xffffffffu;
constexpr int kSeg = 16;  // steps between checkpoints (and per recomputed segment)
constexpr int kCalibBlock = 64;

template <typename T>
struct CalibScale;
template <>
struct CalibScale<float> {
    static __device__ float init(int H) { return ldexpf(1.f, 120) / (float)H; }
    static constexpr double log10_scale = 36.12359947967774;
};
template <>
struct CalibScale<double> {
    static __device__ double init(int H) { return ldexp(1.0, 1020) / (double)H; }
    static constexpr double log10_scale = 307.0505955772608;
};

template <typename T>
__device__ __forceinline__ T pow10_(float x);
template <>
__device__ __forceinline__ float pow10_<float>(float x) { return exp10f(x); }
template <>
__device__ __forceinline__ double pow10_<double>(float x) { return exp10((double)x); }

// Row coefficients (a=MM, b=IM, e=MI, f=II, h=MD, k=DD) and priors of one lane's rows.
template <typename T, int K>
struct Rows {
    T a[K], b[K], e[K], f[K], h[K], k[K], pm[K], pe[K];
    T eo[K], ec[K];  // 10^g, 10^c (for the parameter gradients)
    uint32_t rb[K];  // read base (0x100: dummy row, matches nothing)
};

template <typename T, int K>
__device__ __forceinline__ void load_rows(const DevTables &TB, const ghmm_calib_batch &in, int64_t roff, int R, int pad,
                                          int lane, Rows<T, K> &w) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const int p = lane * K + k - pad;
        if (p < 0) {
            w.a[k] = w.b[k] = w.e[k] = w.f[k] = w.h[k] = (T)0;
            w.k[k] = (T)1;
            w.pm[k] = w.pe[k] = (T)0;
            w.eo[k] = w.ec[k] = (T)0;
            w.rb[k] = 0x100u;
        } else {
            const T eo = pow10_<T>(in.gap_open[roff + p]);
            const T ec = pow10_<T>(in.gap_cont[roff + p]);
            const uint8_t q = in.quals[roff + p], base = in.bases[roff + p];
            w.eo[k] = eo;
            w.ec[k] = ec;
            w.a[k] = (T)1 - (T)2 * eo;
            w.b[k] = (T)1 - ec;
            w.e[k] = eo;
            w.h[k] = eo;
            w.f[k] = ec;
            w.k[k] = ec;
            w.pm[k] = (T)__ldg(TB.prob_d + q);
            w.pe[k] = base == 'N' ? w.pm[k] : (T)__ldg(TB.err3_d + q);
            w.rb[k] = base;
        }
    }
}

template <typename T>
__device__ __forceinline__ T prior_of(uint32_t rb, uint32_t y, T pm, T pe) {
    return (rb == y || y == 'N') ? pm : pe;
}

// Warp front: each lane's rows after its last step plus the diagonal inputs of the next step.
template <typename T, int K>
struct Front {
    T M[K], I[K], D[K];
    T gM, gI, gD;
};

// One forward step; returns the "up" values (row above at this lane's column) through uM/uI/uD.
// pad: dummy rows above the strip's first row (the read's top padding in strip 0, <= 0 in later strips); bnd: the
// previous strip's last row (M, I, D per column), or NULL in strip 0 (row 0: M = I = 0, D = scale / H).
template <typename T, int K>
__device__ __forceinline__ void fwd_step(const Rows<T, K> &w, Front<T, K> &f, const uint8_t *hb, int H, int s, int lane,
                                         int pad, T init, const T *bnd, T &uM, T &uI, T &uD) {
    const int c = s - lane;
    const bool valid = c >= 0 && c < H;
    const uint32_t y = valid ? (uint32_t)hb[c] : 0x200u;
    uM = __shfl_up_sync(kFullMask, f.M[K - 1], 1);
    uI = __shfl_up_sync(kFullMask, f.I[K - 1], 1);
    uD = __shfl_up_sync(kFullMask, f.D[K - 1], 1);
    if (c == 0) {  // column-0 boundary
#pragma unroll
        for (int k = 0; k < K; ++k) {
            f.M[k] = f.I[k] = (T)0;
            f.D[k] = (lane * K + k < pad) ? init : (T)0;
        }
        f.gM = f.gI = (T)0;
        f.gD = (lane * K - 1 < pad) ? init : (T)0;
    }
    if (lane == 0) {
        if (!bnd) {  // row 0: M = I = 0, D = scale / H
            uM = (T)0;
            uI = (T)0;
            uD = init;
        } else {  // the previous strip's last row at this column
            uM = valid ? bnd[3 * c + 0] : (T)0;
            uI = valid ? bnd[3 * c + 1] : (T)0;
            uD = valid ? bnd[3 * c + 2] : (T)0;
        }
    }
#pragma unroll
    for (int k = K - 1; k >= 0; --k) {
        const T dM = k ? f.M[k - 1] : f.gM, dI = k ? f.I[k - 1] : f.gI, dD = k ? f.D[k - 1] : f.gD;
        const T pr = prior_of<T>(w.rb[k], y, w.pm[k], w.pe[k]);
        const T Mn = pr * (dM * w.a[k] + (dI + dD) * w.b[k]);
        const T Dn = f.M[k] * w.h[k] + f.D[k] * w.k[k];
        f.M[k] = Mn;
        f.D[k] = Dn;
    }
    T aM = uM, aI = uI;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        const T In = aM * w.e[k] + aI * w.f[k];
        f.I[k] = In;
        aM = f.M[k];
        aI = In;
    }
    f.gM = uM;
    f.gI = uI;
    f.gD = uD;
}

// scratch layout per warp (all T): checkpoints [nck][3K+3][32], segment fronts [kSeg][3K+3][32], the strips' last
// rows [nstrips - 1][H][3] (forward), and two buffers [H][4] of first-row adjoint values (backward, by strip parity)
template <typename T, int K>
__device__ __forceinline__ void save_front(T *dst, const Front<T, K> &f, int lane) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
        dst[(3 * k + 0) * 32 + lane] = f.M[k];
        dst[(3 * k + 1) * 32 + lane] = f.I[k];
        dst[(3 * k + 2) * 32 + lane] = f.D[k];
    }
    dst[(3 * K + 0) * 32 + lane] = f.gM;
    dst[(3 * K + 1) * 32 + lane] = f.gI;
    dst[(3 * K + 2) * 32 + lane] = f.gD;
}
template <typename T, int K>
__device__ __forceinline__ void load_front(const T *src, Front<T, K> &f, int lane) {
#pragma unroll
    for (int k = 0; k < K; ++k) {
        f.M[k] = src[(3 * k + 0) * 32 + lane];
        f.I[k] = src[(3 * k + 1) * 32 + lane];
        f.D[k] = src[(3 * k + 2) * 32 + lane];
    }
    f.gM = src[(3 * K + 0) * 32 + lane];
    f.gI = src[(3 * K + 1) * 32 + lane];
    f.gD = src[(3 * K + 2) * 32 + lane];
}

// MULTI: reads may need more than one strip (K = 8 batches with reads longer than 256 bases); otherwise every read fits
// one strip and the strip logic folds away.
template <typename T, int K, bool BACKWARD, bool MULTI>
__device__ void calib_pair(const DevTables &TB, const ghmm_calib_batch &in, int64_t pair, T *scratch, double *loglik,
                           const double *weights, float *grad_open, float *grad_cont, int *need_fp64, bool fp64_pass) {
    constexpr int F = 3 * K + 3;  // values per lane in a front
    const int lane = threadIdx.x & 31;
    const int read = in.pair_read[pair], hap = in.pair_hap[pair];
    const int64_t roff = in.read_off[read];
    const int R = (int)(in.read_off[read + 1] - roff);
    const int64_t hoff = in.hap_off[hap];
    const int H = (int)(in.hap_off[hap + 1] - hoff);
    if (R == 0 || H == 0) {
        if (lane == 0) loglik[pair] = -INFINITY;
        return;
    }
    constexpr int S = 32 * K;
    const int nstrips = MULTI ? (R + S - 1) / S : 1;
    const int pad0 = nstrips * S - R;  // dummy rows above the read, in strip 0
    const uint8_t *hb = in.hap_bases + hoff;
    const T init = CalibScale<T>::init(H);
    const int nsteps = H + 31;
    const int nseg = (nsteps + kSeg - 1) / kSeg;
    T *seg = scratch + (size_t)nseg * F * 32;
    T *fwd_bnd = seg + (size_t)kSeg * F * 32;                 // [nstrips - 1][H][3]
    T *adj_bnd = fwd_bnd + (size_t)(nstrips - 1) * H * 3;     // [2][H][4]
    Rows<T, K> w;
    Front<T, K> f;
    // forward, strip by strip; checkpoints of the strip being run (the last strip's stay for its backward)
    T acc = (T)0;
    for (int st = 0; st < nstrips; ++st) {
        const int pad = pad0 - st * S;
        const T *bnd = st ? fwd_bnd + (size_t)(st - 1) * H * 3 : nullptr;
        T *bnd_out = fwd_bnd + (size_t)st * H * 3;
        load_rows<T, K>(TB, in, roff, R, pad, lane, w);
#pragma unroll
        for (int k = 0; k < K; ++k) f.M[k] = f.I[k] = f.D[k] = (T)0;
        f.gM = f.gI = f.gD = (T)0;
        for (int s = 0; s < nsteps; ++s) {
            if (BACKWARD && s % kSeg == 0) save_front<T, K>(scratch + (size_t)(s / kSeg) * F * 32, f, lane);
            T uM, uI, uD;
            fwd_step<T, K>(w, f, hb, H, s, lane, pad, init, bnd, uM, uI, uD);
            const int c = s - lane;
            if (lane == 31 && c >= 0 && c < H) {
                if (st == nstrips - 1) {
                    acc += f.M[K - 1] + f.I[K - 1];
                } else {
                    bnd_out[3 * c + 0] = f.M[K - 1];
                    bnd_out[3 * c + 1] = f.I[K - 1];
                    bnd_out[3 * c + 2] = f.D[K - 1];
                }
            }
        }
        __syncwarp();
    }
    const T Ls = __shfl_sync(kFullMask, acc, 31);
    const bool under = !(Ls >= (T)GHMM_FP32_RERUN_THRESHOLD) || !(Ls <= (T)FLT_MAX);
    if (!fp64_pass && under) {  // FP32 underflow: the FP64 pass redoes this pair
        if (lane == 0) need_fp64[pair] = 1;
        return;
    }
    if (lane == 0) loglik[pair] = log10((double)Ls) - CalibScale<T>::log10_scale;
    if (!BACKWARD) return;

    // ---------------- backward, strips last to first ----------------
    const T seed = (T)weights[pair] / Ls;
    for (int st = nstrips - 1; st >= 0; --st) {
        const int pad = pad0 - st * S;
        const T *bnd = st ? fwd_bnd + (size_t)(st - 1) * H * 3 : nullptr;
        const bool last = st == nstrips - 1;
        // the first-row adjoints of the strip below (read by lane 31) and of this strip (written by lane 0)
        const T *adj_in = adj_bnd + (size_t)((st + 1) & 1) * H * 4;
        T *adj_out = adj_bnd + (size_t)(st & 1) * H * 4;
        if (!last) {  // this strip's checkpoints: its forward again, from the row above it
            load_rows<T, K>(TB, in, roff, R, pad, lane, w);
#pragma unroll
            for (int k = 0; k < K; ++k) f.M[k] = f.I[k] = f.D[k] = (T)0;
            f.gM = f.gI = f.gD = (T)0;
            for (int s = 0; s < nsteps; ++s) {
                if (s % kSeg == 0) save_front<T, K>(scratch + (size_t)(s / kSeg) * F * 32, f, lane);
                T uM, uI, uD;
                fwd_step<T, K>(w, f, hb, H, s, lane, pad, init, bnd, uM, uI, uD);
            }
            __syncwarp();
        }
        // adjoint state of this lane's rows at the previous reverse step (column c+1)
        T gam[K], bI[K], bD[K];
        T Ga[K], Gb[K], Ge[K], Gf[K], Gh[K], Gk[K];
#pragma unroll
        for (int k = 0; k < K; ++k) {
            gam[k] = bI[k] = bD[k] = (T)0;
            Ga[k] = Gb[k] = Ge[k] = Gf[k] = Gh[k] = Gk[k] = (T)0;
        }
        T dgA = (T)0, dgB = (T)0;  // from the row below: a*gamma, b*gamma of its first row at column c+1
        T snA = (T)0, snB = (T)0, snE = (T)0, snF = (T)0;  // what this lane sent last reverse step
        const bool below = lane != 31 || !last;  // lane 31 of the last strip holds the read's last row
        for (int sg = nseg - 1; sg >= 0; --sg) {
            const int s0 = sg * kSeg, s1 = min(s0 + kSeg, nsteps);
            // recompute the segment's fronts (front after each step, plus the step's "up" values)
            Front<T, K> r;
            load_front<T, K>(scratch + (size_t)sg * F * 32, r, lane);
            for (int s = s0; s < s1; ++s) {
                T uM, uI, uD;
                fwd_step<T, K>(w, r, hb, H, s, lane, pad, init, bnd, uM, uI, uD);
                T *dst = seg + (size_t)(s - s0) * F * 32;
                save_front<T, K>(dst, r, lane);  // gM/gI/gD slots now hold this step's up values
            }
            __syncwarp();
            for (int s = s1 - 1; s >= s0; --s) {
                const int c = s - lane;
                const bool valid = c >= 0 && c < H;
                // below (row under this lane's last row) at column c, and its a*gamma, b*gamma for column c: from
                // lane l+1, or for lane 31 from the first row of the strip below
                T inE = __shfl_down_sync(kFullMask, snE, 1), inF = __shfl_down_sync(kFullMask, snF, 1);
                T inA = __shfl_down_sync(kFullMask, snA, 1), inB = __shfl_down_sync(kFullMask, snB, 1);
                if (lane == 31) {
                    const bool have = !last && valid;
                    inE = have ? adj_in[4 * c + 0] : (T)0;
                    inF = have ? adj_in[4 * c + 1] : (T)0;
                    inA = have ? adj_in[4 * c + 2] : (T)0;
                    inB = have ? adj_in[4 * c + 3] : (T)0;
                }
                // forward values: column c (after step s) and c-1 (after step s-1)
                Front<T, K> cur, prv;
                load_front<T, K>(seg + (size_t)(s - s0) * F * 32, cur, lane);
                if (s > s0) {
                    load_front<T, K>(seg + (size_t)(s - 1 - s0) * F * 32, prv, lane);
                } else {
                    load_front<T, K>(scratch + (size_t)sg * F * 32, prv, lane);  // checkpoint = front before step s0
                    // the checkpoint's gM/gI/gD are the diagonal inputs of step s0 = up values of step s0-1
                }
                if (c == 0) {  // the forward used the column-0 boundary as left and diagonal inputs here
#pragma unroll
                    for (int k = 0; k < K; ++k) {
                        prv.M[k] = prv.I[k] = (T)0;
                        prv.D[k] = (lane * K + k < pad) ? init : (T)0;
                    }
                    prv.gM = prv.gI = (T)0;
                    prv.gD = (lane * K - 1 < pad) ? init : (T)0;
                }
                // up values of step s (row above at column c) and diagonal (column c-1)
                const T upM = cur.gM, upI = cur.gI;
                const T dgM = prv.gM, dgI = prv.gI, dgD = prv.gD;
                const uint32_t y = valid ? (uint32_t)hb[c] : 0x200u;
                const bool last_lane = lane == 31;
                T newGam[K], newBI[K], newBD[K];
                T belowE = below ? inE : (T)0, belowF = below ? inF : (T)0;  // e,f of row below times its betaI
                T diagA = below ? dgA : (T)0, diagB = below ? dgB : (T)0;    // a,b of row below times gamma(c+1)
#pragma unroll
                for (int k = K - 1; k >= 0; --k) {
                    T seedM = (T)0;
                    if (last && last_lane && k == K - 1) seedM = seed;
                    const T bD_new = diagB + w.k[k] * bD[k];
                    const T bI_new = seedM + diagB + belowF;
                    const T bM = seedM + diagA + belowE + w.h[k] * bD[k];
                    const T pr = prior_of<T>(w.rb[k], y, w.pm[k], w.pe[k]);
                    T g = pr * bM;
                    T bi = bI_new, bd = bD_new;
                    if (!valid) g = bi = bd = (T)0;
                    newGam[k] = g;
                    newBI[k] = bi;
                    newBD[k] = bd;
                    // forward neighbours of cell (row k, column c)
                    const T mUp = k ? cur.M[k - 1] : upM, iUp = k ? cur.I[k - 1] : upI;
                    const T mDg = k ? prv.M[k - 1] : dgM, iDg = k ? prv.I[k - 1] : dgI, dDg = k ? prv.D[k - 1] : dgD;
                    Ga[k] += g * mDg;
                    Gb[k] += g * (iDg + dDg);
                    Ge[k] += bi * mUp;
                    Gf[k] += bi * iUp;
                    Gh[k] += bd * prv.M[k];
                    Gk[k] += bd * prv.D[k];
                    // for the row above (k-1) in this lane: this row's coefficients times its adjoints
                    belowE = w.e[k] * bi;
                    belowF = w.f[k] * bi;
                    diagA = w.a[k] * gam[k];  // gamma of this row at column c+1 (previous reverse step)
                    diagB = w.b[k] * gam[k];
                }
#pragma unroll
                for (int k = 0; k < K; ++k) {
                    gam[k] = newGam[k];
                    bI[k] = newBI[k];
                    bD[k] = newBD[k];
                }
                // what the row above needs: row 0's e,f * betaI at column c (used now) and a,b * gamma at column c
                snE = w.e[0] * bI[0];
                snF = w.f[0] * bI[0];
                snA = w.a[0] * gam[0];
                snB = w.b[0] * gam[0];
                if (lane == 0 && st > 0 && valid) {  // for lane 31 of the strip above
                    adj_out[4 * c + 0] = snE;
                    adj_out[4 * c + 1] = snF;
                    adj_out[4 * c + 2] = snA;
                    adj_out[4 * c + 3] = snB;
                }
                dgA = inA;  // the row below's a*gamma at column c becomes the diagonal input of column c-1
                dgB = inB;
            }
            __syncwarp();
        }
        // per-row parameter gradients of this strip: d(w log10 L)/dg and /dc
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const int p = lane * K + k - pad;
            if (p >= 0) {
                const T dg = w.eo[k] * (Ge[k] + Gh[k] - (T)2 * Ga[k]);
                const T dc = w.ec[k] * (Gf[k] + Gk[k] - Gb[k]);
                atomicAdd(grad_open + roff + p, (float)dg);
                atomicAdd(grad_cont + roff + p, (float)dc);
            }
        }
        __syncwarp();
    }
}

template <typename T, int K, bool BACKWARD, bool MULTI>
__global__ void __launch_bounds__(kCalibBlock) calib_kernel(DevTables TB, ghmm_calib_batch in, T *scratch,
                                                            int64_t scratch_per_warp, double *loglik,
                                                            const double *weights, float *grad_open, float *grad_cont,
                                                            int *need_fp64, int fp64_pass) {
    const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
    T *my = scratch + warp * scratch_per_warp;
    for (int64_t p = warp; p < in.n_pairs; p += nwarps) {
        if (fp64_pass && !need_fp64[p]) continue;
        calib_pair<T, K, BACKWARD, MULTI>(TB, in, p, my, loglik, weights, grad_open, grad_cont, need_fp64,
                                          fp64_pass != 0);
        __syncwarp();
    }
}

// Blocks of one instantiation resident on an SM (from its registers), looked up once per process.
template <typename T, int K, bool BACKWARD, bool MULTI>
int calib_resident_blocks() {
    static std::atomic<int> blocks{0};
    int b = blocks.load(std::memory_order_relaxed);
    if (b == 0) {
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, calib_kernel<T, K, BACKWARD, MULTI>, kCalibBlock, 0) !=
                cudaSuccess ||
            b < 1)
            b = 1;
        blocks.store(b, std::memory_order_relaxed);
    }
    return b;
}

}  // namespace

int64_t calib_scratch_per_warp(int k, int max_hap_len, int max_read_len, bool fp64) {
    const int64_t F = 3 * k + 3;
    const int64_t nsteps = max_hap_len + 31;
    const int64_t fronts = (nsteps + kSeg - 1) / kSeg + kSeg;
    const int64_t nstrips = ((int64_t)max_read_len + 32 * k - 1) / (32 * k);
    const int64_t boundaries = (nstrips - 1) * max_hap_len * 3 + 2 * (int64_t)max_hap_len * 4;
    return (fronts * F * 32 + boundaries) * (fp64 ? 8 : 4);
}

// Six blocks of two warps per SM: 12 warps, what the 154-register FP32 backward at K = 5 keeps resident; on
// 4,096 pairs of 150-base reads and 300-base haplotypes 7 % faster forward + backward than four blocks, and
// faster than eight.  Instantiations
// with fewer resident blocks (the FP64 backward at up to 255 registers) launch only those, so that no block waits
// for a second wave with pairs already assigned to it by the grid stride.
int calib_grid(int sm_count) { return sm_count * 6; }
int calib_block() { return kCalibBlock; }

int launch_calib(const DevTables &TB, const ghmm_calib_batch &in, int k, bool backward, bool fp64, void *scratch,
                 int64_t scratch_bytes_per_warp, double *loglik, const double *weights, float *grad_open,
                 float *grad_cont, int *need_fp64, int grid, int sm_count, cudaStream_t s) {
#define GHMM_CALIB_ONE(T, KK, BWD, MUL)                                                                             \
    calib_kernel<T, KK, BWD, MUL>                                                                                   \
        <<<std::min(grid, sm_count * calib_resident_blocks<T, KK, BWD, MUL>()), kCalibBlock, 0, s>>>(              \
            TB, in, (T *)scratch, scratch_bytes_per_warp / (int64_t)sizeof(T), loglik, weights, grad_open,           \
            grad_cont, need_fp64, fp64 ? 1 : 0)
#define GHMM_CALIB(KK, MUL)                                                                                         \
    if (fp64) {                                                                                                     \
        if (backward)                                                                                               \
            GHMM_CALIB_ONE(double, KK, true, MUL);                                                                  \
        else                                                                                                        \
            GHMM_CALIB_ONE(double, KK, false, MUL);                                                                 \
    } else {                                                                                                        \
        if (backward)                                                                                               \
            GHMM_CALIB_ONE(float, KK, true, MUL);                                                                   \
        else                                                                                                        \
            GHMM_CALIB_ONE(float, KK, false, MUL);                                                                  \
    }
    switch (k) {
        case 1: GHMM_CALIB(1, false) break;
        case 2: GHMM_CALIB(2, false) break;
        case 3: GHMM_CALIB(3, false) break;
        case 4: GHMM_CALIB(4, false) break;
        case 5: GHMM_CALIB(5, false) break;
        case 6: GHMM_CALIB(6, false) break;
        case 7: GHMM_CALIB(7, false) break;
        case 8:
            if (in.max_read_len > 32 * 8) {
                GHMM_CALIB(8, true)
            } else {
                GHMM_CALIB(8, false)
            }
            break;
        default:
            return (int)cudaErrorInvalidValue;
    }
#undef GHMM_CALIB
#undef GHMM_CALIB_ONE
    return (int)cudaGetLastError();
}

}  // namespace ghmm
