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

#ifdef __cplusplus
}
#endif

#endif
