/*
 * ghmm.h -- C-ABI of the GB300-native PairHMM (CUDA_LOGLESS) for GATK's read-likelihood step.
 *
 * The entry points mirror the native PairHMM binding GATK calls through JNI:
 *   org.broadinstitute.gatk.nativebindings.pairhmm.PairHMMNativeBinding (gatk-native-bindings 1.1.0),
 *   used by src/main/java/org/broadinstitute/hellbender/utils/pairhmm/VectorLoglessPairHMM.java:57-168:
 *     boolean load(File)                                   -> ghmm_load          (VectorLoglessPairHMM.java:63,71)
 *     void initialize(PairHMMNativeArguments)              -> ghmm_initialize    (VectorLoglessPairHMM.java:81)
 *     void computeLikelihoods(ReadDataHolder[], HaplotypeDataHolder[], double[])
 *                                                          -> ghmm_compute_likelihoods (VectorLoglessPairHMM.java:138)
 *     void done()                                          -> ghmm_done          (VectorLoglessPairHMM.java:164)
 * ReadDataHolder {readBases, readQuals, insertionGOP, deletionGOP, overallGCP} (VectorLoglessPairHMM.java:122-127)
 * maps to ghmm_read; HaplotypeDataHolder {haplotypeBases} (:97-98) maps to ghmm_hap.
 *
 * Results are log10 likelihoods, read-major: out[r * n_haps + h] (VectorLoglessPairHMM.java:131,147-148),
 * with the semantics of LoglessPairHMM (LoglessPairHMM.java:20-68): an FP32 wavefront with a 2^120-scaled
 * initial condition, and an FP64 rerun (2^1020 scale) for every pair whose FP32 sum falls below
 * GHMM_FP32_RERUN_THRESHOLD or is not finite.
 *
 * Ownership: callers own every input array and `out`; the library copies inputs into its own
 * staging buffers during the call and keeps no caller pointer after it returns.  `out` is fully
 * written before a successful return.
 * Errors: every call returns a status code (GHMM_OK = 0); ghmm_last_error gives the message.
 * Threading: a context is used by one caller thread at a time; separate contexts are independent
 * (each owns its own CUDA stream and buffers), as GATK creates one PairHMM per likelihood engine
 * (HC/PairHMMLikelihoodCalculationEngine.java:145) and one engine per Spark partition.
 */
#ifndef GHMM_H
#define GHMM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes.  The JNI layer maps ERR_UNSUPPORTED to UserException.HardwareFeatureException,
 * ERR_ARG to IllegalArgumentException, ERR_STATE to IllegalStateException, and the rest to
 * GATKException (PairHMM.java:284-306, VectorLoglessPairHMM.java:63-79). */
#define GHMM_OK 0
#define GHMM_ERR_ARG 1         /* invalid argument (lengths, quality bytes out of range, NULL) */
#define GHMM_ERR_STATE 2       /* context not initialised / already done */
#define GHMM_ERR_CUDA 3        /* CUDA runtime error */
#define GHMM_ERR_UNSUPPORTED 4 /* no usable sm_103 GPU */
#define GHMM_ERR_RESULT 5      /* a likelihood was > 0 or NaN (PairHMM.java:305-306) */
#define GHMM_ERR_NOMEM 6       /* device or pinned host allocation failed */
#define GHMM_ERR_TIMEOUT 7     /* a bounded device-side wait ran out */

/* FP32 scaled-sum threshold below which a pair is recomputed in FP64.  The FP32 sum carries the
 * 2^120 scale, so 1e-28 means log10 L < -64.1; cells on the dominant alignment path are then still
 * ten decades above FLT_MIN (1.18e-38), where gradual underflow would start to cost precision. */
#define GHMM_FP32_RERUN_THRESHOLD 1e-28f

/* The FP64 path has two tiers: a rescaled recurrence (5 DP operations per cell, scale 2^960) for every pair,
 * and LoglessPairHMM's unscaled recurrence (scale 2^1020) for pairs whose rescaled result falls below
 * log10 L = GHMM_FP64_RESCALED_FLOOR or is not finite, so results near the bottom of the FP64 range, and
 * -Infinity, come out as the reference computes them. */
#define GHMM_FP64_RESCALED_FLOOR (-560.0)

/* Forward modes for ghmm_batch_forward. */
#define GHMM_MODE_PD 3         /* PD-HMM batch (ghmm_pd_batch_create): every pair in the FP64 PD-HMM kernel */
#define GHMM_MODE_PD_FP32 4    /* PD-HMM batch: FP32 PD-HMM kernel (scale 2^120) + FP64 rerun of underflowing pairs;
                                  ghmm_pd_compute_* use it unless the context is double precision */
#define GHMM_MODE_FP32_RERUN 0 /* batched FP32 wavefront + FP64 rerun of underflowing pairs (default) */
#define GHMM_MODE_FP64 1       /* every pair in the FP64 wavefront kernel (useDoublePrecision) */
#define GHMM_MODE_PLAIN_FP64 2 /* plain FP64 kernel, one pair per thread block, one launch per region; reads <= 2048 */

/* Mirrors PairHMMNativeArguments {maxNumberOfThreads, useDoublePrecision}
 * (HC/PairHMMNativeArgumentCollection.java:11-23) plus the device to use. */
typedef struct ghmm_args {
    int32_t device;               /* CUDA device ordinal */
    int32_t max_threads;          /* host threads used to marshal inputs (<= 0: all cores) */
    int32_t use_double_precision; /* nonzero: every pair in FP64 (GHMM_MODE_FP64) */
    int32_t flags;                /* reserved, must be 0 */
} ghmm_args;

/* ReadDataHolder: five arrays of `length` bytes; quals are Phred values (not +33). */
typedef struct ghmm_read {
    const uint8_t *bases;
    const uint8_t *quals;
    const uint8_t *ins_gop;
    const uint8_t *del_gop;
    const uint8_t *gcp;
    int32_t length;
} ghmm_read;

/* HaplotypeDataHolder */
typedef struct ghmm_hap {
    const uint8_t *bases;
    int32_t length;
} ghmm_hap;

/* One active region: its reads against its haplotypes (one computeLikelihoods call). */
typedef struct ghmm_region {
    const ghmm_read *reads;
    int32_t n_reads;
    const ghmm_hap *haps;
    int32_t n_haps;
} ghmm_region;

/* The same inputs already laid out as flat planes (int64 offsets), as ghmm_synth produces. */
typedef struct ghmm_flat {
    int64_t n_regions;
    const int64_t *region_read_off; /* [n_regions+1] */
    const int64_t *region_hap_off;  /* [n_regions+1] */
    const int64_t *read_off;        /* [n_reads+1] byte offsets into the five planes */
    const uint8_t *bases, *quals, *ins_gop, *del_gop, *gcp;
    const int64_t *hap_off;         /* [n_haps+1] byte offsets into hap_bases */
    const uint8_t *hap_bases;
    const int64_t *out_off;         /* [n_regions+1] read-major block offsets into out */
} ghmm_flat;

typedef struct ghmm_ctx ghmm_ctx;
typedef struct ghmm_batch ghmm_batch;
typedef struct ghmm_queue ghmm_queue;

/* Per-batch statistics (filled by ghmm_batch_stats after ghmm_batch_forward). */
typedef struct ghmm_stats {
    int64_t n_pairs;          /* read x haplotype pairs */
    int64_t n_cells;          /* sum over pairs of read_len * hap_len */
    int64_t n_rerun;          /* pairs recomputed in FP64 after the FP32 pass */
    int64_t n_fp64_direct;    /* pairs sent to FP64 directly (gcp 0, non-ACGTN bytes, FP64 mode) */
    int64_t n_tasks_fp32;     /* warp tasks of the FP32 pass */
    int32_t n_launches;       /* kernels launched by the last forward */
    int32_t reserved;
    double ms_fp32;           /* device time of the FP32 launches (CUDA events), last forward */
    double ms_fp64;           /* device time of the FP64 rerun / FP64-mode launches */
    double ms_plain;          /* device time of the plain FP64 launches */
    double ms_total;          /* device time of the whole forward */
    int64_t h2d_bytes;        /* host-to-device bytes of the last upload + forward */
    int64_t d2h_bytes;        /* device-to-host bytes of the last forward + results */
    double ms_host_marshal;   /* host time of the last marshal: copies into pinned planes, checks, routing */
    double ms_host_tasks;     /* host time of building and ordering the FP32 warp tasks */
    int64_t n_fp64_exact;     /* pairs of the last forward computed by the exact (unscaled, 2^1020) FP64 tier:
                                 results of the rescaled FP64 tier below log10 L = -560, and host-marked reads */
    double ms_prep;           /* raw batches: device time of the read preparation kernels of the upload (quality
                                 caps, PCR model or DRAGstr imputation); 0 for prepared batches */
    int64_t n_cells_fp64_direct; /* cells of the pairs the last forward sent to FP64 without an FP32 pass */
} ghmm_stats;

/* Launch-shape choices of the FP32 pass (the autotuner's knobs; the reference has none besides its thread
 * count).  A read of R bases runs single-strip with ceil(R/32) rows per lane when that is at most
 * max_rows_per_lane, otherwise as the fewest strips of at most max_rows_per_lane_multi rows per lane.
 * route_fp64_below sends a read's pairs to the FP64 kernel without an FP32 pass when the read's expected
 * log10 prior product -- the sum over its positions of (1 - e) log10(1 - e) + e log10(e / 3), e the base
 * error probability -- is below it: such pairs would fall under GHMM_FP32_RERUN_THRESHOLD (log10 L < -64)
 * and be recomputed in FP64 anyway.  Results are the same either way (the FP64 result of a pair does not
 * depend on how it reached the FP64 kernel); only time changes.  The autotuner keeps it as set.
 * Zero fields keep their defaults (8, 8, 16384, -100). */
typedef struct ghmm_tuning {
    int32_t max_rows_per_lane;       /* 1..8 */
    int32_t max_rows_per_lane_multi; /* 1..8 */
    int32_t chunk_cols;              /* haplotype columns per FP32 task, >= 1 */
    int32_t route_fp64_below;        /* log10 units, < 0; -1000000 in effect turns the routing off */
} ghmm_tuning;

/* PairHMMNativeBinding.load: 1 if a usable GPU (compute capability 10.3) is present, else 0. */
int ghmm_load(void);

/* PairHMMNativeBinding.initialize: create a context on args->device. */
int ghmm_initialize(const ghmm_args *args, ghmm_ctx **ctx);

/* PairHMMNativeBinding.computeLikelihoods: out[r * n_haps + h] for one region (read-major). */
int ghmm_compute_likelihoods(ghmm_ctx *ctx, const ghmm_read *reads, int32_t n_reads, const ghmm_hap *haps,
                             int32_t n_haps, double *out);

/* Set the FP32 launch shape used by batches created after this call (see ghmm_tuning). */
int ghmm_set_tuning(ghmm_ctx *ctx, const ghmm_tuning *tuning);
int ghmm_get_tuning(ghmm_ctx *ctx, ghmm_tuning *tuning);

/* Autotuner (no counterpart in the reference, which has no launch shape to choose): time every candidate
 * tuning on a sample of the caller's workload -- marshal with that tuning, one warm-up forward, then the
 * median device time of reps forwards (0: 3) -- set the fastest on ctx and return it in *best.
 * candidates NULL / n_candidates 0 selects the built-in grid: max_rows_per_lane {8, 6, 4} x
 * max_rows_per_lane_multi {8, 6, 4} x chunk_cols {16384, 4096}, in that order; ms (may be NULL) receives
 * each candidate's median milliseconds.  The sample should hold a few times 1e10 cells. */
int ghmm_autotune(ghmm_ctx *ctx, const ghmm_flat *sample, const ghmm_tuning *candidates, int32_t n_candidates,
                  int32_t reps, ghmm_tuning *best, double *ms);

/* PairHMMNativeBinding.done: release the context. */
int ghmm_done(ghmm_ctx *ctx);

/* Message of the last failed call on ctx (or of the last failed ghmm_initialize when ctx is NULL). */
int ghmm_last_error(const ghmm_ctx *ctx, char *buf, size_t buf_len);

/* Batcher: many regions in one call (regions of HaplotypeCallerEngine.callRegion batched together).
 * out receives each region's read-major block back to back, in region order.  Inputs of 1.5e11 cells or
 * more run as a pipeline of batches (the first small, later ones up to a third of the input) on the
 * context's internal queue, so that marshalling overlaps the kernels; the results are the same. */
int ghmm_compute_regions(ghmm_ctx *ctx, const ghmm_region *regions, int32_t n_regions, double *out);

/* Device-resident batches: marshal + upload once, run the forward many times, download. */
int ghmm_batch_create(ghmm_ctx *ctx, const ghmm_region *regions, int32_t n_regions, ghmm_batch **batch);
int ghmm_batch_create_flat(ghmm_ctx *ctx, const ghmm_flat *flat, ghmm_batch **batch);
int ghmm_batch_forward(ghmm_ctx *ctx, ghmm_batch *batch, int32_t mode);
int ghmm_batch_results(ghmm_ctx *ctx, ghmm_batch *batch, double *out);
int ghmm_batch_stats(ghmm_ctx *ctx, const ghmm_batch *batch, ghmm_stats *stats);
int ghmm_batch_destroy(ghmm_ctx *ctx, ghmm_batch *batch);

/* The step after the likelihoods, fused on the device over a batch's last forward: per read, every haplotype
 * likelihood below best + cap is raised to best + cap (AlleleLikelihoods.normalizeLikelihoods,
 * utils/genotyper/AlleleLikelihoods.java:416-458, best as searchBestAllele :505-540), and reads whose best
 * likelihood is below their threshold are flagged for removal (filterPoorlyModeledEvidence :1351-1376 with
 * ReadLikelihoodCalculationEngine.log10MinTrueLikelihood :124-132, or the DRAGEN-GATK dynamic threshold
 * :106-158), in that order, as PairHMMLikelihoodCalculationEngine.java:200-201 runs them.  The normalised values
 * replace the batch's results (ghmm_batch_results); keep[r] (n_reads bytes, host) is 1 for a read that stays.
 * One region is one sample and its haplotypes are the alleles. */
typedef struct ghmm_postprocess {
    double max_likelihood_difference_cap; /* log10globalReadMismappingRate: < 0, or -INFINITY to skip normalising */
    int32_t symmetric;                    /* symmetricallyNormalizeAllelesToReference: the reference may be best */
    int32_t dynamic_disqualification;     /* dynamicDisqualification: the DRAGEN-GATK read-quality threshold */
    double expected_error_rate_per_base;  /* expectedErrorRatePerBase (GATK default 0.02), >= 0 */
    double read_disqualification_scale;   /* readDisqualificationScale (GATK default 1.0) */
    const int32_t *reference_hap;         /* per region: reference haplotype index within the region or -1; NULL: none */
} ghmm_postprocess;

int ghmm_batch_postprocess(ghmm_ctx *ctx, ghmm_batch *batch, const ghmm_postprocess *pp, uint8_t *keep);

/* Flat inputs straight from host memory to results (upload + forward + download in one call). */
int ghmm_compute_flat(ghmm_ctx *ctx, const ghmm_flat *flat, double *out);

/* The CUDA stream the context launches on (a cudaStream_t), for callers that time or order work. */
void *ghmm_stream(ghmm_ctx *ctx);

/* Reads as they come off the alignment, prepared for the PairHMM on the device: what
 * PairHMMLikelihoodCalculationEngine.modifyReadQualities does on the host in GATK (HC/PairHMMLikelihoodCalculation
 * Engine.java:283-322): the PCR indel error model (:331-371, with findTandemRepeatUnits,
 * HC/ReadLikelihoodCalculationEngine.java:193-253), base qualities capped by the mapping quality, base qualities below
 * the threshold and insertion / deletion qualities below 6 set to 6; and the standard input-score imputation (a
 * constant gap continuation penalty; insertion / deletion qualities from the BI / BD tags, or 45 when a read has
 * none, ReadUtils.java:838-862).  Soft-clip removal stays with the caller (it needs the CIGAR). */
typedef struct ghmm_raw_read {
    const uint8_t *bases;
    const uint8_t *quals;     /* base qualities as read */
    const uint8_t *ins_quals; /* BI tag, or NULL for 45 */
    const uint8_t *del_quals; /* BD tag, or NULL for 45 */
    int32_t length;
    int32_t mapping_quality;
} ghmm_raw_read;

typedef struct ghmm_raw_region {
    const ghmm_raw_read *reads;
    int32_t n_reads;
    const ghmm_hap *haps;
    int32_t n_haps;
} ghmm_raw_region;

/* DRAGEN-GATK's STR-aware imputation (DragstrPairHMMInputScoreImputator.impute, HC/DragstrPairHMMInputScoreImputator
 * .java:54-88): at every read position but the last, the most repeated short tandem repeat period around it and its
 * repeat count (DragstrReadSTRAnalyzer, PH/DragstrReadSTRAnalyzer.java, periods 1..max_period, ties to the shorter
 * period) index the model's tables (DragstrParams.gop / gcp, utils/dragstr/DragstrParams.java:194-220: periods and
 * repeats beyond the table use its last row / column); the insertion and deletion open penalties are
 * Math.round(min(40, gop)) and the continuation penalty Math.round(gcp), as Java bytes; the last position gets 45 and
 * 10. */
typedef struct ghmm_dragstr {
    int32_t max_period;  /* DragstrParams.maximumPeriod(), 1..32 */
    int32_t max_repeats; /* DragstrParams.maximumRepeats(), >= 1 */
    const double *gop;   /* [max_period][max_repeats]: gop(period, repeats) at [period - 1][repeats - 1] */
    const double *gcp;   /* same layout */
} ghmm_dragstr;

typedef struct ghmm_read_prep {
    int32_t base_quality_threshold; /* --base-quality-score-threshold (PairHMM.BASE_QUALITY_SCORE_THRESHOLD = 18) */
    int32_t cap_to_mapq;            /* !disableCapReadQualitiesToMapQ */
    double pcr_rate_factor;         /* PCRErrorModel: 0 NONE, 1 HOSTILE, 2 AGGRESSIVE, 3 CONSERVATIVE (GATK default) */
    int32_t gcp;                    /* constant gap continuation penalty (--gcp-hmm, default 10), 1..127 */
    int32_t reserved;
    const ghmm_dragstr *dragstr;    /* NULL: the standard imputation above; else the DRAGstr imputation, which
                                     * replaces the insertion / deletion / continuation penalties (the PCR model and
                                     * the floor of 6 then do not apply to them) */
} ghmm_read_prep;

/* As ghmm_compute_regions, from raw reads; the preparation runs on the device before the forward. */
int ghmm_compute_regions_raw(ghmm_ctx *ctx, const ghmm_raw_region *regions, int32_t n_regions, const ghmm_read_prep *prep,
                             double *out);
int ghmm_batch_create_raw(ghmm_ctx *ctx, const ghmm_raw_region *regions, int32_t n_regions, const ghmm_read_prep *prep,
                          ghmm_batch **batch);
/* Copy a batch's five read planes as the kernels see them (after the device preparation of a raw batch) into
 * host arrays of n_read_bytes each, reads back to back in batch order; any pointer may be NULL. */
int ghmm_batch_read_planes(ghmm_ctx *ctx, const ghmm_batch *batch, uint8_t *bases, uint8_t *quals, uint8_t *ins,
                           uint8_t *dels, uint8_t *gcp);

/* Partially-determined-haplotype PairHMM (PD-HMM), the DRAGEN-GATK mode's likelihood step: LoglessPDPairHMM
 * (PH/LoglessPDPairHMM.java:35-150), whose native binding IntelPDHMM.computeLikelihoods(ReadDataHolder[],
 * HaplotypeDataHolder[], double[]) is called at PH/VectorLoglessPairPDHMM.java:98.  A PD haplotype carries, beside its
 * bases, one flag byte per base (PartiallyDeterminedHaplotype.java:59-66: SNP 1, DEL_START 2, DEL_END 4, and the
 * alternative-base bits A 8, C 16, G 32, T 64, N 128), HaplotypeDataHolder.haplotypePDBases.  Results are read-major
 * as ghmm_compute_likelihoods.  ghmm_pd_compute_* run GHMM_MODE_PD_FP32 (FP32 at scale 2^120, pairs whose sums
 * underflow recomputed in FP64), or GHMM_MODE_PD (FP64 at the reference's 2^1020 scale for every pair) when the
 * context is double precision, as the regular path does.  A read base other than A, C, G, T (either
 * case) or N that meets an undetermined SNP column is an argument error, where the reference throws
 * ("Found unexpected base in alt alleles", LoglessPDPairHMM.java:196-210). */
typedef struct ghmm_pd_hap {
    const uint8_t *bases;
    const uint8_t *pd_bases; /* flag byte per base */
    int32_t length;
    int32_t reserved;
} ghmm_pd_hap;

typedef struct ghmm_pd_region {
    const ghmm_read *reads;
    int32_t n_reads;
    const ghmm_pd_hap *haps;
    int32_t n_haps;
} ghmm_pd_region;

int ghmm_pd_compute_likelihoods(ghmm_ctx *ctx, const ghmm_read *reads, int32_t n_reads, const ghmm_pd_hap *haps,
                                int32_t n_haps, double *out);
int ghmm_pd_compute_regions(ghmm_ctx *ctx, const ghmm_pd_region *regions, int32_t n_regions, double *out);
/* A device-resident PD batch; run it with ghmm_batch_forward(..., GHMM_MODE_PD or GHMM_MODE_PD_FP32). */
int ghmm_pd_batch_create(ghmm_ctx *ctx, const ghmm_pd_region *regions, int32_t n_regions, ghmm_batch **batch);

/* The PD-HMM from raw reads, prepared on the device as ghmm_compute_regions_raw prepares them: the DRAGEN-GATK
 * mode's chain of DRAGstr imputation (ghmm_read_prep.dragstr) and PD-HMM likelihoods in one call. */
typedef struct ghmm_pd_raw_region {
    const ghmm_raw_read *reads;
    int32_t n_reads;
    const ghmm_pd_hap *haps;
    int32_t n_haps;
} ghmm_pd_raw_region;

int ghmm_pd_compute_regions_raw(ghmm_ctx *ctx, const ghmm_pd_raw_region *regions, int32_t n_regions,
                                const ghmm_read_prep *prep, double *out);
int ghmm_pd_batch_create_raw(ghmm_ctx *ctx, const ghmm_pd_raw_region *regions, int32_t n_regions,
                             const ghmm_read_prep *prep, ghmm_batch **batch);

/* Streaming queue: regions enqueued one at a time as they arrive, as HaplotypeCaller produces them.
 * No counterpart in the reference's binding, whose computeLikelihoods is synchronous per active region
 * (PH/VectorLoglessPairHMM.java:138, called once per region from HC/HaplotypeCallerEngine.java:734-918
 * through PairHMMLikelihoodCalculationEngine.computeReadLikelihoods); the queue is what a caller puts in
 * front of it to batch regions.
 *   ghmm_queue_create: a queue on ctx; batches are launched once they hold batch_cells cells (0: 2e11).
 *   ghmm_queue_push:   copy n_regions regions into the open batch before returning, so the caller may
 *                      reuse its arrays; their read-major results go to out (as ghmm_compute_regions), which
 *                      must stay valid until ghmm_queue_flush returns.  Input errors are reported by this
 *                      call and leave the queue unchanged; an error of an earlier batch (a device failure or
 *                      an invalid result) is returned by every later push and flush.
 *   ghmm_queue_flush:  launch the open batch and wait until every pushed region's results are in place.
 *   ghmm_queue_get_info: totals over the queue's finished batches.
 *   ghmm_queue_destroy: flush, then release the queue (before ghmm_done of its context).
 * A worker thread marshals and launches full batches on two streams with two buffer slots.  One queue is
 * driven by one thread at a time; ghmm_set_tuning is refused while a queue is open. */
typedef struct ghmm_queue_info {
    int64_t n_regions;            /* regions pushed */
    int64_t n_pairs;              /* read x haplotype pairs pushed */
    int64_t n_cells;              /* cells pushed */
    int64_t n_cells_fp64_direct;  /* cells of finished pairs sent to FP64 directly (the rest ran in FP32) */
    int64_t n_rerun;              /* finished pairs recomputed in FP64 after the FP32 pass */
    int64_t n_fp64_direct;        /* finished pairs sent to FP64 directly */
    int64_t n_batches;            /* batches finished */
    int64_t n_launches;           /* kernels launched by the finished batches */
    int64_t h2d_bytes, d2h_bytes; /* bytes copied by the finished batches */
    double ms_fp32, ms_fp64;      /* summed device time of the two phases (batches on the two streams overlap) */
    double ms_host_marshal;       /* summed worker time in marshalling copies and checks */
    double ms_host_tasks;         /* summed worker time in building FP32 tasks */
    int64_t n_fp64_exact;         /* finished pairs computed by the exact FP64 tier */
} ghmm_queue_info;

int ghmm_queue_create(ghmm_ctx *ctx, int64_t batch_cells, ghmm_queue **queue);
int ghmm_queue_push(ghmm_queue *queue, const ghmm_region *regions, int32_t n_regions, double *out);
int ghmm_queue_flush(ghmm_queue *queue);
int ghmm_queue_get_info(ghmm_queue *queue, ghmm_queue_info *info);
int ghmm_queue_destroy(ghmm_queue *queue);

/* A queue of raw reads, prepared on the device batch by batch (as ghmm_compute_regions_raw prepares them):
 *   ghmm_queue_create_raw: prep (checked as ghmm_compute_regions_raw checks it, DRAGstr tables copied) applies to
 *                          every batch of the queue;
 *   ghmm_queue_push_raw:   as ghmm_queue_push, for raw regions.
 * A raw queue takes only ghmm_queue_push_raw, a queue from ghmm_queue_create only ghmm_queue_push
 * (GHMM_ERR_STATE otherwise).  Flush, info and destroy are shared. */
int ghmm_queue_create_raw(ghmm_ctx *ctx, int64_t batch_cells, const ghmm_read_prep *prep, ghmm_queue **queue);
int ghmm_queue_push_raw(ghmm_queue *queue, const ghmm_raw_region *regions, int32_t n_regions, double *out);

/* Failure injection for tests, all on the host side (nothing faults, traps or stalls a GPU):
 *   GHMM_INJECT_REFUSE_ALLOCATIONS: the next arg device allocations of the process fail as out of memory, so the
 *                                   calls that need them return GHMM_ERR_NOMEM and the context stays usable;
 *   GHMM_INJECT_FP64_RERUN_EVERY:   every arg-th output of the FP32 pass is treated as an underflow and recomputed
 *                                   in FP64 (batches uploaded after the call; 0 turns it off).
 * Setting the environment variable GHMM_REPORT_UNSUPPORTED (not "0") makes ghmm_load report no usable GPU, as a
 * caller's fallback chain sees it (VectorLoglessPairHMM.java:60-79 -> HardwareFeatureException). */
#define GHMM_INJECT_REFUSE_ALLOCATIONS 1
#define GHMM_INJECT_FP64_RERUN_EVERY 2
int ghmm_debug_inject(ghmm_ctx *ctx, int32_t kind, int64_t arg);

/* Measured FP32 FMA-pipe peak of the device in TFLOP/s (FMA = 2 FLOP): best of a scalar FFMA and a
 * packed FFMA2 register-resident loop over all SMs, timed with CUDA events.  Also reports the FP64
 * DFMA peak.  Either output may be NULL. */
int ghmm_measure_peaks(ghmm_ctx *ctx, double *fp32_tflops, double *fp32x2_tflops, double *fp64_tflops);

/* Debug/test: copy the context's device-side lookup tables back (double versions):
 * err[256] = 10^(-q/10), prob[256] = 1 - err, m2m[128*128] = matchToMatchProb(ins, del).
 * With ctx == NULL the host-built tables are returned (no device needed). */
int ghmm_debug_tables(ghmm_ctx *ctx, double *err, double *prob, double *m2m);

/* Debug/test (no device needed): the per-column op bytes of the packed FP32 PD-HMM kernel for one haplotype of H
 * bases with PD flags (PartiallyDeterminedHaplotype bits) into ops[H] -- bit 0: copy the branch states; 1: an
 * AFTER_DEL column; 2: a DEL_END column; 3: the next column is AFTER_DEL; 4: an undetermined SNP, its alternative in
 * bits 5-6 (A, C, G, T = 0..3); 7 (with 4): three bases match, bits 5-6 name the fourth -- and the column base codes
 * that kernel reads into codes[H] (A, C, G, T, N = 0..4; an SNP column whose alternatives cover all four bases reads
 * as N).  Returns 1 when the packed kernel takes the haplotype (its row-end state is NORMAL), 0 when its pairs go to
 * the general PD kernel, GHMM_ERR_ARG for bad arguments. */
int ghmm_debug_pd_ops(const uint8_t *bases, const uint8_t *pd_flags, int32_t H, uint8_t *ops, uint8_t *codes);

/* Debug/test (no device needed): the chunks a pipelined call cuts regions of these cells into (ghmm_compute_regions,
 * _flat and _raw on inputs of 1.5e11 cells or more; the one-shot PD-HMM calls on every input): cuts[0] = 0 <
 * cuts[1] < ... = n_regions, chunk i being regions [cuts[i], cuts[i + 1]).  Below 5e11 cells the cuts fall where
 * the running sum of cells first reaches 1/8 and 1/2 of the total; from 5e11, the first chunk takes 1/16 of the cells
 * and each next one 2.5 times the last, up to 1/3.  No cut leaves fewer than 8 regions behind it.  Writes
 * min(cap, *n_cuts) entries; GHMM_ERR_ARG for a negative count or cell number or a NULL array. */
int ghmm_debug_pipeline_cuts(const int64_t *cells, int64_t n_regions, int64_t *cuts, int64_t cap, int64_t *n_cuts);

/* ---- Several devices from one caller ----
 * One handle drives several GPUs (HaplotypeCaller's one JVM; the reference parallelises the host side with GKL's
 * thread count, HC/PairHMMNativeArgumentCollection.java:11-12, or one engine per Spark partition,
 * tools/HaplotypeCallerSpark.java:175-179).  The handle owns one context per device.  A call's reads, numbered
 * in region order, are cut into one contiguous range per device carrying about equal cells (read length x the
 * summed lengths of its region's haplotypes); a contiguous read range owns a contiguous slice of the read-major
 * `out`, so each device writes its results straight into its slice.  No device-to-device traffic, no collective.
 *   ghmm_multi_create:           a context per listed device (devices may repeat: independent contexts on one
 *                                GPU); args as ghmm_initialize, device ignored, max_threads <= 0 shares the host
 *                                cores between the devices.  Setting the environment variable
 *                                GHMM_MULTI_STUB_DEVICES (not "0") creates host-only stand-ins that subtract
 *                                (index + 1) over their slice of `out` instead of computing, so the split can be
 *                                tested without a GPU.
 *   ghmm_multi_compute_regions:  as ghmm_compute_regions over all devices, one host thread per device.
 *   ghmm_multi_plan:             the split alone (host only): slices[d] for n_devices devices.
 *   ghmm_multi_context:          the context of device index `index` (for tuning, statistics, batches).
 *   ghmm_multi_last_error / ghmm_multi_destroy. */
typedef struct ghmm_multi ghmm_multi;

typedef struct ghmm_multi_slice {
    int64_t read_begin, read_end; /* reads of the call, numbered across regions in order: [read_begin, read_end) */
    int64_t out_begin, out_end;   /* the slice of out those reads' likelihoods fill */
    int64_t cells;                /* cells of the slice */
} ghmm_multi_slice;

int ghmm_multi_create(const int32_t *devices, int32_t n_devices, const ghmm_args *args, ghmm_multi **multi);
int ghmm_multi_compute_regions(ghmm_multi *multi, const ghmm_region *regions, int32_t n_regions, double *out);
int ghmm_multi_plan(const ghmm_region *regions, int32_t n_regions, int32_t n_devices, ghmm_multi_slice *slices);
int ghmm_multi_context(ghmm_multi *multi, int32_t index, ghmm_ctx **ctx);
int ghmm_multi_last_error(const ghmm_multi *multi, char *buf, size_t buf_len);
int ghmm_multi_destroy(ghmm_multi *multi);

/* ---- No-allocation entry point.  It has no counterpart in the reference. ----
 * For callers that cannot allocate GPU memory (code running inside another framework's memory pool or
 * a fixed device-memory budget, or that must not take the synchronisation an allocation implies):
 * log10 likelihoods of explicit (read, haplotype) pairs whose bytes the caller already holds in device
 * memory, written to d_out[n_pairs] (device), with the FP64 wavefront kernel.  The call allocates
 * nothing: its scratch (strip-boundary rows for reads longer than 128 bases, 12 MiB) and its Phred
 * tables are static device arrays that every GPU which loads the library holds until the process exits.
 * The first call on a device (made with that device current) resolves the scratch address, fills the
 * tables and waits for them to land (a device synchronisation, once), so it should come before any stream
 * capture.  Calls share the scratch array, which keeps the last call's contents, and must not overlap on
 * the GPU: overlapping calls race on it.  Haplotypes longer than GHMM_NOALLOC_MAX_HAP_LEN are rejected
 * with GHMM_ERR_ARG (max_hap_len is the caller's bound; a longer haplotype found on the device yields NaN
 * for its pair).  The input bytes live on the device, so they are checked there: a pair whose read has a
 * base quality above 254 or an insertion, deletion or gap-continuation penalty above 127 (a negative Java
 * byte) yields NaN, where the other entry points return GHMM_ERR_ARG.  Launches on `stream` (a
 * cudaStream_t; NULL is the legacy default stream) and returns without waiting; the caller's current
 * device is left as it was.  Error messages come from ghmm_last_error(NULL, ...). */
#define GHMM_NOALLOC_MAX_HAP_LEN 2048
#define GHMM_NOALLOC_WARPS 256

typedef struct ghmm_dev_pairs {
    const uint8_t *bases, *quals, *ins_gop, *del_gop, *gcp; /* device read planes */
    const int64_t *read_off;                                /* device [n_reads+1] */
    const uint8_t *hap_bases;                               /* device */
    const int64_t *hap_off;                                 /* device [n_haps+1] */
    const int32_t *pair_read, *pair_hap;                    /* device [n_pairs] */
    int64_t n_pairs;
    int32_t max_hap_len; /* caller's bound on every haplotype length, <= GHMM_NOALLOC_MAX_HAP_LEN */
    int32_t reserved;
} ghmm_dev_pairs;

int ghmm_forward_pairs_noalloc(int32_t device, const ghmm_dev_pairs *pairs, double *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif
