/*
 * ghmm_sw.h -- C-ABI of the GB300 Smith-Waterman aligner: the step after the read likelihoods, where
 * HaplotypeCaller and Mutect2 realign every read to its best haplotype.
 *
 * The single-alignment entry point mirrors the native aligner binding GATK calls through JNI:
 *   org.broadinstitute.gatk.nativebindings.smithwaterman.SWAlignerNativeBinding (gatk-native-bindings 1.1.0),
 *   wrapped by src/main/java/org/broadinstitute/hellbender/utils/smithwaterman/SWNativeAlignerWrapper.java:
 *     boolean load(File)                       -> ghmm_load / ghmm_initialize  (SmithWatermanIntelAligner.java:31-35)
 *     SWNativeAlignerResult align(byte[] ref, byte[] alt, SWParameters, SWOverhangStrategy)
 *                                              -> ghmm_sw_align                (SWNativeAlignerWrapper.java:53)
 *     void close()                             -> ghmm_done                    (SWNativeAlignerWrapper.java:67)
 * SWNativeAlignerResult {String cigar; int alignment_offset} is the text cigar (htsjdk TextCigarCodec) and the
 * offset.  Results are those of SmithWatermanJavaAligner (SmithWatermanJavaAligner.java:59-379) bit for bit:
 * the same int32 scores, gap-length bookkeeping, tie-breaking, end-cell choice per overhang strategy and
 * traceback.
 *
 * Two batched entry points have no counterpart in the binding, whose align is one pair per JNI call:
 *   ghmm_sw_align_batch  many (ref, alt) pairs with one parameter set and strategy, optionally with the exact-
 *                        substring shortcut that SWNativeAlignerWrapper.align:37-50 and SmithWatermanJavaAligner.
 *                        align:71-84 apply before aligning (an alt found in the ref aligns as alt_len M at the
 *                        rightmost match, Utils.lastIndexOf, for SOFTCLIP and IGNORE);
 *   ghmm_batch_realign   AssemblyBasedCallerUtils.realignReadsToTheirBestHaplotype (:107-121) up to the aligner
 *                        call of AlignmentUtils.createReadAlignedToRef (:67): per read of a PairHMM batch that has
 *                        run a forward, the best haplotype of its region by AlleleLikelihoods.
 *                        bestAllelesBreakingTies (searchBestAllele with tie-breaking priorities,
 *                        AlleleLikelihoods.java:505-560, 1062-1075) over the batch's current likelihoods, then the
 *                        read aligned against it with SOFTCLIP and the substring shortcut.  The sequences and the
 *                        likelihoods stay on the GPU; only the cigars come back.  What createReadAlignedToRef does
 *                        with the cigar afterwards (mapping through the haplotype's cigar, left-aligning indels)
 *                        stays with the caller.
 * Batched cigars come back BAM-encoded (length << 4 | op, op M 0, I 1, D 2, S 4), each alignment's ops
 * contiguous in one caller array.  2 * alt_len + 4 ops bound any one alignment.
 *
 * Errors: ref or alt empty or NULL -> GHMM_ERR_ARG with SmithWatermanJavaAligner's message
 * (SmithWatermanJavaAligner.java:65-67); NULL parameters or an unknown strategy -> GHMM_ERR_ARG.
 */
#ifndef GHMM_SW_H
#define GHMM_SW_H

#include <stddef.h>
#include <stdint.h>

#include "ghmm.h"

#ifdef __cplusplus
extern "C" {
#endif

/* SWOverhangStrategy */
#define GHMM_SW_SOFTCLIP 0
#define GHMM_SW_INDEL 1
#define GHMM_SW_LEADING_INDEL 2
#define GHMM_SW_IGNORE 3

/* flags of ghmm_sw_align_batch */
#define GHMM_SW_SUBSTRING_SHORTCUT 1

/* BAM cigar operator codes of the batched results */
#define GHMM_CIGAR_M 0
#define GHMM_CIGAR_I 1
#define GHMM_CIGAR_D 2
#define GHMM_CIGAR_S 4

/* Longest ref or alt accepted */
#define GHMM_SW_MAX_LEN (1 << 20)

/* SWParameters(matchValue, mismatchPenalty, gapOpenPenalty, gapExtendPenalty); GATK's sets are in
 * SmithWatermanAlignmentConstants.java:30-68, e.g. ALIGNMENT_TO_BEST_HAPLOTYPE_SW_PARAMETERS = {10, -15, -30, -5}. */
typedef struct ghmm_sw_params {
    int32_t match_value;
    int32_t mismatch_penalty;
    int32_t gap_open_penalty;
    int32_t gap_extend_penalty;
} ghmm_sw_params;

typedef struct ghmm_sw_pair {
    const uint8_t *ref;
    const uint8_t *alt;
    int32_t ref_len;
    int32_t alt_len;
} ghmm_sw_pair;

/* Results of n alignments.  Alignment i's ops are cigar_ops[cigar_start[i] .. cigar_start[i] + cigar_len[i]). */
typedef struct ghmm_sw_result {
    int32_t *alignment_offset; /* [n] SWNativeAlignerResult.alignment_offset (-1: not aligned, see realign) */
    int64_t *cigar_start;      /* [n] */
    int32_t *cigar_len;        /* [n] */
    uint32_t *cigar_ops;       /* [cigar_cap] */
    int64_t cigar_cap;         /* capacity of cigar_ops; GHMM_ERR_ARG when the cigars need more */
    int64_t cigar_total;       /* out: ops written */
} ghmm_sw_result;

/* Timings and counts of the last Smith-Waterman call on a context. */
typedef struct ghmm_sw_stats {
    int64_t n_alignments;  /* pairs (or reads) of the call */
    int64_t n_shortcut;    /* solved by the exact-substring shortcut */
    int64_t cells;         /* ref_len x alt_len summed over the alignments that ran the score recurrence */
    int32_t chunks;        /* passes over the traceback buffer */
    int32_t launches;      /* kernels launched */
    double ms_device;      /* device time of the kernels (CUDA events), without the host planning between phases */
    double ms_forward;     /* summed time of the score-recurrence kernels */
    double ms_total;       /* wall time of the call */
    int64_t h2d_bytes, d2h_bytes;
    double ms_host;        /* host time: checks, marshalling, chunk and task planning */
    int64_t n_int16;       /* alignments run two per warp in 16-bit halves (the rest in int32) */
} ghmm_sw_stats;

/* SWAlignerNativeBinding.align: the cigar as text into cigar[cigar_cap] (NUL-terminated; GHMM_ERR_ARG when
 * it does not fit) and the alignment offset.  Like the native binding, no substring shortcut (the Java wrapper
 * applies it before calling the binding). */
int ghmm_sw_align(ghmm_ctx *ctx, const uint8_t *ref, int32_t ref_len, const uint8_t *alt, int32_t alt_len,
                  const ghmm_sw_params *params, int32_t strategy, char *cigar, int32_t cigar_cap,
                  int32_t *alignment_offset);

/* Sum of 2 * alt_len + 4 over the pairs: a cigar_cap that always suffices. */
int64_t ghmm_sw_cigar_bound(const ghmm_sw_pair *pairs, int32_t n_pairs);

int ghmm_sw_align_batch(ghmm_ctx *ctx, const ghmm_sw_pair *pairs, int32_t n_pairs, const ghmm_sw_params *params,
                        int32_t strategy, int32_t flags, ghmm_sw_result *result);

/* hap_priority: one value per haplotype of the batch (batch order), the tie-breaking priority of
 * AssemblyBasedCallerUtils.HAPLOTYPE_ALIGNMENT_TIEBREAKING_PRIORITY (:65-70: 1 for the reference haplotype plus
 * 1 - the number of elements of the haplotype's cigar), or NULL for no tie-breaking.  Outputs per read of the
 * batch: best_hap (index within its region; -1 for a region without haplotypes, whose reads are not aligned and
 * get alignment_offset -1), informative (BestAllele.isInformative), and the alignment in result (cigar_cap of
 * 2 * (read bytes) + 4 * reads always suffices). */
int ghmm_batch_realign(ghmm_ctx *ctx, ghmm_batch *batch, const double *hap_priority, const ghmm_sw_params *params,
                       int32_t *best_hap, uint8_t *informative, ghmm_sw_result *result);

int ghmm_sw_last_stats(ghmm_ctx *ctx, ghmm_sw_stats *stats);

/* Device memory for traceback bits (4 bits per cell, in 32-bit words per lane and step); by default 16 GiB or a
 * quarter of the device memory free when the context first aligns, whichever is less.  A
 * call whose alignments need more runs in several passes over the buffer; a single alignment larger than the
 * budget gets a pass of its own.  Values below 1 MiB are raised to 1 MiB. */
int ghmm_sw_set_traceback_budget(ghmm_ctx *ctx, int64_t bytes);

/* Kernel choice.  By default alignments whose scores provably fit in 16 bits (bounded by the sequence lengths and
 * parameters) run two per warp in the 16-bit halves of each register, the rest in int32; results are identical.
 * GHMM_SW_OPT_INT32_ONLY runs everything in int32. */
#define GHMM_SW_OPT_INT32_ONLY 1
int ghmm_sw_set_options(ghmm_ctx *ctx, int32_t flags);

/* Measured int32 max/compare throughput of the device in Tops/s: a register-resident loop of independent max.s32
 * chains over all SMs, timed with CUDA events.  The roofline denominator of the score recurrence, whose cells are
 * adds, compares and maxima. */
int ghmm_sw_measure_peak(ghmm_ctx *ctx, double *int32_tops);

#ifdef __cplusplus
}
#endif

#endif
