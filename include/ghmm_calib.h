/*
 * ghmm_calib.h -- gap-penalty calibration entry points of the GB300 PairHMM (DRAGstr model).
 *
 * GATK's DRAGstr mode sets each read position's gap-open and gap-continuation penalties from the
 * short tandem repeat it sits in (DragstrPairHMMInputScoreImputator.java:54-88 with
 * DragstrParams.java:194-220 and DragstrReadSTRAnalyzer.java:110-136).  These entry points expose the
 * STR analysis and a differentiable forward/backward PairHMM over a (period, repeat) parameter table,
 * so the penalties can be fitted by maximum likelihood.  The reference has no gradient; the analysis
 * mirrors DragstrReadSTRAnalyzer.
 */
#ifndef GHMM_CALIB_H
#define GHMM_CALIB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* DragstrReadSTRAnalyzer.of(bases, maxPeriod): for every position i, best_period[i] =
 * mostRepeatedPeriod(i) (DragstrReadSTRAnalyzer.java:110) and best_repeats[i] = numberOfMostRepeats(i)
 * (:133); all_repeats (may be NULL) receives numberOfRepeats(i, p) at [(p-1)*n + i] (:92).
 * Returns 0 on success. */
int ghmm_str_analyze(const uint8_t *bases, int32_t n, int32_t max_period, int32_t *best_period,
                     int32_t *best_repeats, int32_t *all_repeats);

typedef struct ghmm_ctx ghmm_ctx;

/* A calibration batch, all arrays in device memory owned by the caller.  For every read position p the
 * gap-open and gap-continuation log10-probabilities g = gap_open[p], c = gap_cont[p] define the row's
 * transitions MI = MD = 10^g, MM = 1 - 2*10^g, II = DD = 10^c, IM = 1 - 10^c (the continuous form of
 * PairHMMModel.qualToTransProbs, PairHMMModel.java:107-117); priors come from the base qualities
 * (LoglessPairHMM.java:79-93). */
typedef struct ghmm_calib_batch {
    const uint8_t *bases, *quals;        /* read planes (quals are Phred values) */
    const int64_t *read_off;             /* [n_reads+1] */
    const uint8_t *hap_bases;
    const int64_t *hap_off;              /* [n_haps+1] */
    const int32_t *pair_read, *pair_hap; /* [n_pairs] */
    const float *gap_open, *gap_cont;    /* per read position, indexed like the read planes */
    int64_t n_pairs;
    int32_t max_read_len;                /* 1..65536: one strip up to 256 bases, strips of 256 rows beyond */
    int32_t max_hap_len;
} ghmm_calib_batch;

/* log10 L of every pair into d_loglik[n_pairs] (device).  precision 0: FP32 (scale 2^120) with an FP64 redo
 * of pairs whose FP32 likelihood underflows (below 1e-28 scaled); 1: FP64 throughout (scale 2^1020). */
int ghmm_calib_forward(ghmm_ctx *ctx, const ghmm_calib_batch *batch, int32_t precision, double *d_loglik);

/* Forward and hand-written backward.  d_loglik as above; d_grad_open / d_grad_cont (device, one float per
 * read position, accumulated into, so zero them first) receive sum_p w_p * d log10 L_p / d g (resp. c) with
 * w_p = d_weights[p] (device, NULL: all ones).  The forward is recomputed from checkpoints every 16 wavefront
 * steps during the backward sweep; reads longer than 256 bases run in strips of 256 rows, whose boundary rows
 * (forward) and first-row adjoints (backward) pass through per-warp scratch, the backward taking the strips last
 * to first.  The context holds that scratch (for the forward too when reads exceed 256 bases): at most
 * GHMM_CALIB_SCRATCH_BYTES bytes (environment, read at each call; default 4 GiB), launching fewer warps, each
 * taking more pairs, where long pairs would need more for a full grid. */
int ghmm_calib_backward(ghmm_ctx *ctx, const ghmm_calib_batch *batch, int32_t precision, const double *d_weights,
                        double *d_loglik, float *d_grad_open, float *d_grad_cont);

#ifdef __cplusplus
}
#endif

#endif
