// ghmm_internal.h -- device-side data layout shared by the kernels (kernels.cu) and the host runtime
// (runtime.cpp).  Plain C structs: pointers are device addresses.
#pragma once

#include <cstdint>

#include "../../include/ghmm_calib.h"

namespace ghmm {

// Column-stream byte of a haplotype base (one per haplotype column, haplotypes of a region back to
// back): bits 0-2 base index (A=0 C=1 G=2 T=3 N=4), bit 6 first column of a haplotype, bit 7 last.
constexpr uint8_t kColFirst = 0x40;
constexpr uint8_t kColLast = 0x80;
constexpr int kMaxK32 = 8;      // FP32 kernel: rows per lane (strip = 32*K rows)
constexpr int kMaxK64 = 4;      // FP64 kernel: rows per lane
constexpr int kMaxReadLen = 1 << 20;
constexpr int kNumBucketKeys = 32;       // bucket key = rows per lane (1..8) | 16 for multi-strip
constexpr int kCounterBucketBase = 8;    // counters[8 + key]: bucket task cursors
constexpr int kNumCounters = 64;
constexpr int kMaxHapLen = 1 << 20;

// Device lookup tables (QualityUtils / PairHMMModel restated on the host, uploaded once per context).
struct DevTables {
    const float *err_f;     // [256] 10^(-q/10)
    const float *prob_f;    // [256] 1 - 10^(-q/10)
    const float *err3_f;    // [256] 10^(-q/10) / 3
    const float *m2m_f;     // [128*128] matchToMatchProb(ins, del), row = ins
    const double *err_d;
    const double *prob_d;
    const double *err3_d;
    const double *m2m_d;
    const double *lm2m_d;   // [128*128] -log2(m2m_f), the FP32 pass's row rescaling exponent
};

// Read-pair task of the FP32 pass: two reads of one region (b < 0: single read) against the
// haplotypes [hap_begin, hap_end) of that region, in K-row-per-lane strips.
struct F32Task {
    int32_t read_a, read_b;
    int32_t hap_begin, hap_end;
    int32_t region;
    int16_t nstrips, k;
    int32_t pad_a, pad_b;  // dummy rows on top of strip 0 (strip rows * nstrips - read length)
};

// One (read, haplotype) pair for the FP64 kernel.
struct PairRef {
    int32_t read, hap;
};

struct DevBatch {
    // reads: five planes, byte offsets
    const uint8_t *bases, *quals, *ins, *dels, *gcp;
    const int64_t *read_off;
    // haplotypes
    const uint8_t *hap_bases;   // raw bytes
    const uint8_t *hap_code;    // column-stream codes (same indexing as hap_bases)
    const int64_t *hap_off;
    const float *hap_init_f;    // 2^120 / H
    const double *hap_init_d;   // 2^1020 / H
    // regions
    const int64_t *region_read_off, *region_hap_off, *out_off;
    const int32_t *read_region; // region of each read
    double *out;
    // FP32 tasks (all buckets, contiguous per K)
    const F32Task *tasks;
    // FP64 queue: entries [0, n_direct) filled by the host, the rest appended by the FP32 pass
    PairRef *rerun;
    int32_t *counters;          // [1] FP64 queue tail, [2] FP64 cursor, [3] error flag, [8 + key] bucket cursors
    const int32_t *bucket_info; // [key] first task of bucket key, [kNumBucketKeys + key] its task count
    const int64_t *n_out_dev;   // number of outputs (for the FP64 epilogue)
    int64_t rerun_capacity;
    int64_t force_rerun_every;  // test hook (ghmm_debug_inject): every n-th output of the FP32 pass goes to FP64; 0 off
    // strip-boundary scratch of multi-strip FP32 tasks: per resident warp, max_cols float2 x 3
    float2 *scratch32;
    int64_t scratch32_cols;
    double *scratch64;          // FP64 multi-strip boundary: per resident warp, max_hap_len x 3 doubles
    int64_t scratch64_cols;
    const float2 *read_scale;   // per read: (2^-(la - n), n) with la = log2 a_R of the FP32 pass, n = round(la)
};

// Kernel launchers (kernels.cu).  All return cudaError_t as int.
int launch_fp32_bucket(const DevTables &t, const DevBatch &b, int key, int grid, int block, cudaStream_t s);
int launch_fp64_queue(const DevTables &t, const DevBatch &b, int grid, int block, cudaStream_t s);
int launch_finalize_fp32(double *out, const int64_t *n_out, int sm_count, cudaStream_t s);
// Per-read log2 a_R of the FP32 pass (kernels.cu), into scale[n_reads]; after the read planes are final.
int launch_read_scale(const DevTables &t, const DevBatch &b, int64_t n_reads, float2 *scale, int sm_count,
                      cudaStream_t s);
int launch_plain_region(const DevTables &t, const DevBatch &b, int region, int n_reads, int n_haps, int max_read_len,
                        cudaStream_t s);
constexpr int kPlainMaxRead = 2048;
// Rows below each read in the FP32 layout that accumulate the haplotype sum (kernels.cu).
constexpr int kAccRows = 2;
// Zero bytes on both sides of the column-code plane, so the FP32 kernel may load a code one step ahead
// (and lanes that have not started may load before the first column) without leaving the allocation.
constexpr int kCodePad = 64;
// Largest insertion-state growth bound G (I~ <= G max M~) the rescaled FP64 tier takes (headroom 2^60; the bound is a
// worst case, and a pair whose rescaled states do overflow sums to a non-finite value and moves to the exact tier, so
// this only keeps pairs that would almost surely overflow from running twice).
constexpr double kMaxGrowth64 = 1e15;
int fp32_kernel_occupancy(int k, int block, int *blocks_per_sm);
int fp64_kernel_occupancy(int block, int *blocks_per_sm);

// PD-HMM (pd.cu): per haplotype column, the PD flag byte (PartiallyDeterminedHaplotype bits) and the HMM state
// code: bits 0-1 the state the read's first row uses at this column, bits 2-3 the state of the other rows
// (0 NORMAL, 1 INSIDE_DEL, 2 AFTER_DEL), bit 4 this column carries DEL_END.
struct PdPlanes {
    const uint8_t *flags;
    const uint8_t *states;
    const uint8_t *ops;  // per column the packed FP32 kernel's op byte, indexed like hap_code (kCodePad zeros around)
};
// Op bits of the packed FP32 PD kernel (pd_packed.cu), derived per haplotype column by the host (pd_host.cpp).
constexpr uint32_t kPdOpCopy = 1;       // a later column reads this column's branch state: store it (NORMAL: bX =
                                        // previous X; AFTER_DEL: bX = max(bX, previous X))
constexpr uint32_t kPdOpAfter = 2;      // AFTER_DEL column
constexpr uint32_t kPdOpDelEnd = 4;     // DEL_END column: I reads max(bX, X) of the row above
constexpr uint32_t kPdOpNextAfter = 8;  // the next column is AFTER_DEL
constexpr uint32_t kPdOpSnp = 16;       // undetermined SNP: its alternative in bits 5-6 (A, C, G, T = 0..3)
constexpr int kPdOpAltShift = 5;
constexpr uint32_t kPdOpSnpAllBut = 128;  // with kPdOpSnp: three bases match, bits 5-6 name the fourth
// FP32 PD read-pair tasks of bucket key (2..8 rows per lane, | 16 for multi-strip tasks) from the batch's task list.
int launch_pd_bucket(const DevTables &t, const DevBatch &b, const uint8_t *ops, int key, int grid, cudaStream_t s);
int pd_bucket_occupancy(int key, int *blocks_per_sm);
int pd_kernel_occupancy(int *blocks_per_sm);
// PD pairs [begin, begin + count) of the pair list (count_dev: the count in device memory), K rows per lane, in
// FP32 (underflows queued for FP64 at rerun[rerun_capacity..)) or FP64; cursor is the counter the warps draw from.
int launch_pd(const DevTables &t, const DevBatch &b, const PdPlanes &p, int k, bool fp32, int begin, int count,
              int cursor, const int32_t *count_dev, int grid, cudaStream_t s);
constexpr int kPdMaxK = 4;          // PD kernel: rows per lane 1..4 in FP64
constexpr int kPdMaxK32 = 8;        // and 1..8 in FP32
constexpr int kCounterPdBase = 40;  // counters[40 + K]: PD FP64 task cursors (inside the 64 counters, above the buckets)
constexpr int kCounterPdRerun = 45;        // PD pairs the FP32 pass queued for FP64
constexpr int kCounterPdRerunCursor = 46;
constexpr int kCounterPdF32Base = 50;      // counters[50 + K]: PD FP32 task cursors (51..58)

// Read preparation on the device (prep.cu).
struct PrepArgs {
    const int32_t *mapq;     // per read
    uint8_t pcr_cache[24];   // PCR indel model quality per repeat length 0..20
    int pcr, cap_to_mapq, threshold;
    // DRAGstr imputation (dragstr != 0): DragstrParams' GOP and GCP tables [max period][max repeats]
    const double *str_gop, *str_gcp;
    int dragstr, str_max_period, str_max_repeats, max_read_len;
};
int launch_prep(const DevBatch &b, int64_t n_reads, const PrepArgs &p, int sm_count, cudaStream_t s);
int launch_dragstr(const DevBatch &b, int64_t n_reads, const PrepArgs &p, int sm_count, cudaStream_t s);
constexpr int kDragstrMaxRead = 28000;  // reads the DRAGstr kernel's shared memory holds (6.4 bytes per base)
constexpr int kDragstrMaxPeriod = 32;

// Post-likelihood normalisation and filtering (post.cu).
struct PostArgs {
    double cap;                   // log10globalReadMismappingRate (< 0)
    double rate;                  // expected error rate per base
    double scale;                 // dynamic threshold's K
    const int32_t *reference_hap; // per region, or nullptr
    int normalize, symmetric, dynamic;
};
int launch_postprocess(const DevBatch &b, int64_t n_reads, const PostArgs &p, uint8_t *keep, int sm_count,
                       cudaStream_t s);
int measure_peaks_device(int sm_count, double *fp32, double *fp32x2, double *fp64, cudaStream_t s);
// Calibration forward/backward (calib.cu).
int64_t calib_scratch_per_warp(int k, int max_hap_len, int max_read_len, bool fp64);
constexpr int kCalibMaxRead = 65536;  // calibration reads: one strip up to 256 bases, strips of 256 rows beyond
int calib_grid(int sm_count);  // blocks of a full grid; a call may launch fewer (scratch budget)
int calib_block();
int launch_calib(const DevTables &TB, const ghmm_calib_batch &in, int k, bool backward, bool fp64, void *scratch,
                 int64_t scratch_bytes_per_warp, double *loglik, const double *weights, float *grad_open,
                 float *grad_cont, int *need_fp64, int grid, int sm_count, cudaStream_t s);
// Smith-Waterman (sw.cu).  Overhang strategies (SWOverhangStrategy) and BAM cigar op codes.
constexpr int kSwSoftclip = 0, kSwIndel = 1, kSwLeadingIndel = 2, kSwIgnore = 3;
constexpr uint32_t kSwOpM = 0, kSwOpI = 1, kSwOpD = 2, kSwOpS = 4;
constexpr int kSwMaxK = 8;  // alt columns per lane; longer alts run in strips of 32 * 8 columns
// Row stride of the last-column lane's scores in the edge array: K rounded up to whole int4s.
#define kSwRowStride(k) ((((k) + 3) / 4) * 4)
// Steps of one strip of a ref of n rows (n + 31), rounded up to whole groups of 4: traceback words are stored in
// groups of 4 consecutive steps per lane (16 contiguous bytes).
#define sw_steps4(n) ((((int64_t)(n) + 34) / 4) * 4)

// One alignment: alt against ref.  Offsets index the ref / alt planes and the chunk's buffers.
struct SwPair {
    int64_t ref_off, alt_off;
    int64_t tb_off;       // first traceback word: strips x sw_steps4(ref_len) steps x 32 lanes; within a strip the word
                          // of step t and lane l is at ((t / 4) * 32 + l) * 4 + t % 4
    int64_t edge_off;     // ref_len rows of the last-column lane's kSwRowStride(k) scores, then the bottom row as
                          // one row of kSwRowStride(k) per lane and strip (a multiple of 4 ints: int4-aligned rows)
    int64_t slot_off;     // 2 * alt_len + 4 cigar ops, written in reverse by the traceback
    int64_t scratch_off;  // strip boundary (score, horizontal gap) per ref row 0..ref_len, multi-strip alts only
    int32_t ref_len, alt_len;
    int32_t k, pad;       // alt columns per lane
};

struct SwArgs {
    const uint8_t *ref_plane, *alt_plane;
    const SwPair *pairs;  // the chunk's pairs; state / offset / n_ops are indexed like them
    uint32_t *tb;
    int *edges;
    int2 *strip_scratch;
    uint32_t *slot;
    int32_t *state;       // 1: solved by the exact-substring shortcut; 0: int32 recurrence; 2 / 3: 16-bit pair, low /
                          // high half (the 16-bit kernel sets them)
    int32_t *offset;      // alignment offset
    int32_t *n_ops;
    int *error;           // set when a traceback overruns its slot (cannot happen for valid input)
    int match, mismatch, open, extend;
    int strategy, indel_edges, shortcut;
    int clamp;            // apply MATRIX_MIN_CUTOFF (0 when the scores provably never reach it)
};
int launch_sw_forward(const SwArgs &a, int k, const int32_t *tasks, int n_tasks, int *cursor, int grid,
                      cudaStream_t s);
int sw_forward_occupancy(int k, int *blocks_per_sm);
// Two single-strip alignments per warp in 16-bit halves (tasks: A, B or -1); only for pairs whose scores the host
// has bounded inside +-24000.  Writes each alignment's traceback words and edges in the int32 kernel's layout.
int launch_sw_pair16(const SwArgs &a, int k, const int2 *tasks, int n_tasks, int *cursor, int grid, cudaStream_t s);
int sw_pair16_occupancy(int k, int *blocks_per_sm);
// The exact-substring shortcut of every alignment (state 1 + offset), or state 0 for all when a.shortcut is 0.
int launch_sw_prepass(const SwArgs &a, int n_pairs, int sm_count, cudaStream_t s);
int launch_sw_traceback(const SwArgs &a, int n_pairs, cudaStream_t s);
// exclusive scan of the chunk's n_ops into starts (offset by *running, which then advances), gather into ops;
// block_sums: ceil(n_pairs / 1024) int64 of scratch
int launch_sw_compact(const SwArgs &a, int n_pairs, int64_t *starts, int64_t *running, uint32_t *ops, int64_t ops_cap,
                      int64_t *block_sums, cudaStream_t s);

// Read-to-best-haplotype realignment setup (sw.cu): per read, the best haplotype of its region by
// AlleleLikelihoods.searchBestAllele with tie-breaking priorities, written into the read's SwPair (ref fields).
struct SwRealignArgs {
    const double *priority;  // per batch haplotype, or nullptr
    SwPair *pairs;           // one per read, alt fields and buffer offsets filled by the host
    int32_t *best;           // per read: best haplotype's index within its region
    uint8_t *informative;    // per read: BestAllele.isInformative()
    int64_t first_read, n_reads;
};
int launch_sw_realign_setup(const DevBatch &b, const SwRealignArgs &a, int sm_count, cudaStream_t s);
// Measured int32 max throughput of the device in Tops/s (sw.cu).
int measure_int32_peak(int sm_count, double *tops, cudaStream_t s);
// Message returned by ghmm_last_error(NULL, ...) (runtime.cpp).
void set_global_error(const char *msg);

}  // namespace ghmm
