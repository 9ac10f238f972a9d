/*
 * ghmm_synth.h -- deterministic synthetic active-region workloads for the PairHMM.
 *
 * This is benchmark and test input generation; it has no counterpart in the reference
 * (GATK's PairHMM consumes reads and haplotypes produced by assembly).  Workload ids 0-4
 * and their distributions are described at the top of gatk_gb300/csrc/synth.cpp.
 *
 * Layout ("flat workload"), all offsets int64:
 *   region_read_off[n_regions+1], region_hap_off[n_regions+1]  global read / haplotype index ranges
 *   read_off[n_reads+1]   byte offset of each read in the five read planes
 *   bases, quals, ins, dels, gcp   read planes (uint8; quals and penalties are Phred values)
 *   hap_off[n_haps+1], hap_bases   haplotype bytes
 *   out_off[n_regions+1]  offset of each region's read-major n_reads x n_haps block in the output
 */
#ifndef GHMM_SYNTH_H
#define GHMM_SYNTH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ghmm_synth ghmm_synth;

typedef struct ghmm_synth_arrays {
    int64_t n_regions, n_reads, n_haps, read_bytes, hap_bytes, n_out;
    const int64_t *region_read_off, *region_hap_off, *read_off, *hap_off, *out_off;
    const uint8_t *bases, *quals, *ins, *dels, *gcp, *hap_bases;
} ghmm_synth_arrays;

/* Number of regions of the full-size workload (1, 10000, 2000, 512, 100000), or -1. */
int64_t ghmm_synth_default_regions(int32_t workload);

/* Generate regions [region_begin, region_end) of a workload with `threads` host threads
 * (<= 0: all).  Returns 0 on success. */
int ghmm_synth_generate(int32_t workload, uint64_t seed, int64_t region_begin, int64_t region_end, int32_t threads,
                        ghmm_synth **out);

/* Borrow the generated arrays (valid until ghmm_synth_free). */
int ghmm_synth_view(const ghmm_synth *s, ghmm_synth_arrays *arrays);

void ghmm_synth_free(ghmm_synth *s);

#ifdef __cplusplus
}
#endif

#endif
