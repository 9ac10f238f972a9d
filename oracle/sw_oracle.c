/* sw_oracle.c -- CPU restatement of GATK's Smith-Waterman aligner, in C (test infrastructure and the timed CPU
 * baseline of the realignment step; never linked by the product).  The same algorithm as oracle/smithwaterman.py,
 * which the reference's unit-test cases pin.  Follows (paths inside the GATK repository,
 * src/main/java/org/broadinstitute/hellbender/):
 *   SmithWatermanJavaAligner.align / calculateMatrix / calculateCigar
 *       utils/smithwaterman/SmithWatermanJavaAligner.java:59-98, 109-228, 261-379
 *   SWNativeAlignerWrapper.align (exact-substring shortcut :37-50)   utils/smithwaterman/SWNativeAlignerWrapper.java:31-59
 *   Utils.lastIndexOf                                         utils/Utils.java:1124-1138
 * Java int arithmetic wraps at 32 bits: every sum goes through add32.
 * Cigar elements are BAM-encoded: length << 4 | op (M 0, I 1, D 2, S 4).
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

enum { SW_SOFTCLIP = 0, SW_INDEL = 1, SW_LEADING_INDEL = 2, SW_IGNORE = 3 };
enum { OP_M = 0, OP_I = 1, OP_D = 2, OP_S = 4 };

#define MATRIX_MIN_CUTOFF (-100000000)
#define LOW_INIT_VALUE (INT32_MIN / 2)

static inline int32_t add32(int32_t a, int32_t b) { return (int32_t)((uint32_t)a + (uint32_t)b); }

int sw_oracle_last_index_of(const uint8_t *ref, int n, const uint8_t *q, int m) {
    for (int r = n - m; r >= 0; r--) {
        int k = 0;
        while (k < m && ref[r + k] == q[k]) k++;
        if (k == m) return r;
    }
    return -1;
}

typedef struct {
    uint32_t *ops;
    int n, cap, overflow;
} OpList;

static void push(OpList *l, int op, int len) {
    if (l->n < l->cap)
        l->ops[l->n] = ((uint32_t)len << 4) | (uint32_t)op;
    else
        l->overflow = 1;
    l->n++;
}

/* Returns 0, -1 for invalid arguments, -2 when ops_cap is too small, -3 when out of memory. */
int sw_oracle_align(const uint8_t *ref, int ref_len, const uint8_t *alt, int alt_len, const int32_t *params,
                    int strategy, int shortcut, uint32_t *ops, int ops_cap, int32_t *n_ops, int32_t *offset) {
    if (!ref || !alt || ref_len <= 0 || alt_len <= 0 || strategy < 0 || strategy > 3) return -1;
    OpList l = {ops, 0, ops_cap, 0};
    if (shortcut && (strategy == SW_SOFTCLIP || strategy == SW_IGNORE)) {
        const int idx = sw_oracle_last_index_of(ref, ref_len, alt, alt_len);
        if (idx != -1) {
            push(&l, OP_M, alt_len);
            *n_ops = l.n;
            *offset = idx;
            return l.overflow ? -2 : 0;
        }
    }
    const int32_t w_match = params[0], w_mismatch = params[1], w_open = params[2], w_extend = params[3];
    const int64_t n = (int64_t)ref_len + 1, m = (int64_t)alt_len + 1;
    int32_t *sw = (int32_t *)calloc((size_t)(n * m), sizeof(int32_t));
    int32_t *bt = (int32_t *)calloc((size_t)(n * m), sizeof(int32_t));
    int32_t *best_gap_v = (int32_t *)malloc((size_t)(m + 1) * sizeof(int32_t));
    int32_t *gap_size_v = (int32_t *)calloc((size_t)(m + 1), sizeof(int32_t));
    if (!sw || !bt || !best_gap_v || !gap_size_v) {
        free(sw), free(bt), free(best_gap_v), free(gap_size_v);
        return -3;
    }
    for (int64_t j = 0; j <= m; j++) best_gap_v[j] = LOW_INIT_VALUE;
    if (strategy == SW_INDEL || strategy == SW_LEADING_INDEL) {
        int32_t cur = w_open;
        sw[1] = w_open;
        for (int64_t j = 2; j < m; j++) sw[j] = cur = add32(cur, w_extend);
        cur = w_open;
        sw[m] = w_open;
        for (int64_t i = 2; i < n; i++) sw[i * m] = cur = add32(cur, w_extend);
    }
    for (int64_t i = 1; i < n; i++) {
        const uint8_t a = ref[i - 1];
        const int32_t *last = sw + (i - 1) * m;
        int32_t *cur = sw + i * m, *btr = bt + i * m;
        int32_t best_gap_h = LOW_INIT_VALUE, gap_size_h = 0;
        for (int64_t j = 1; j < m; j++) {
            const int32_t step_diag = add32(last[j - 1], a == alt[j - 1] ? w_match : w_mismatch);
            int32_t prev_gap = add32(last[j], w_open);
            best_gap_v[j] = add32(best_gap_v[j], w_extend);
            if (prev_gap > best_gap_v[j]) {
                best_gap_v[j] = prev_gap;
                gap_size_v[j] = 1;
            } else {
                gap_size_v[j]++;
            }
            const int32_t step_down = best_gap_v[j], kd = gap_size_v[j];
            prev_gap = add32(cur[j - 1], w_open);
            best_gap_h = add32(best_gap_h, w_extend);
            if (prev_gap > best_gap_h) {
                best_gap_h = prev_gap;
                gap_size_h = 1;
            } else {
                gap_size_h++;
            }
            const int32_t step_right = best_gap_h, ki = gap_size_h;
            int32_t v;
            if (step_diag >= step_down && step_diag >= step_right) {
                v = step_diag;
                btr[j] = 0;
            } else if (step_right >= step_down) {
                v = step_right;
                btr[j] = -ki;
            } else {
                v = step_down;
                btr[j] = kd;
            }
            cur[j] = v > MATRIX_MIN_CUTOFF ? v : MATRIX_MIN_CUTOFF;
        }
    }
    /* calculateCigar */
    int64_t p1 = 0, p2 = 0;
    int32_t maxscore = INT32_MIN;
    int64_t segment_length = 0;
    const int64_t rl = n - 1, al = m - 1;
    if (strategy == SW_INDEL) {
        p1 = rl;
        p2 = al;
    } else {
        p2 = al;
        for (int64_t i = 1; i < n; i++) {
            const int32_t s = sw[i * m + al];
            if (s >= maxscore) {
                p1 = i;
                maxscore = s;
            }
        }
        if (strategy != SW_LEADING_INDEL) {
            const int32_t *bottom = sw + rl * m;
            for (int64_t j = 1; j < m; j++) {
                const int32_t s = bottom[j];
                const int64_t d_new = rl - j < 0 ? j - rl : rl - j, d_cur = p1 - p2 < 0 ? p2 - p1 : p1 - p2;
                if (s > maxscore || (s == maxscore && d_new < d_cur)) {
                    p1 = rl;
                    p2 = j;
                    maxscore = s;
                    segment_length = al - j;
                }
            }
        }
    }
    /* elements are collected in traceback order and reversed at the end */
    if (segment_length > 0 && strategy == SW_SOFTCLIP) {
        push(&l, OP_S, (int)segment_length);
        segment_length = 0;
    }
    int state = OP_M;
    do {
        const int32_t b = bt[p1 * m + p2];
        int new_state;
        int64_t step = 1;
        if (b > 0) {
            new_state = OP_D;
            step = b;
        } else if (b < 0) {
            new_state = OP_I;
            step = -(int64_t)b;
        } else {
            new_state = OP_M;
        }
        if (new_state == OP_M) {
            p1--;
            p2--;
        } else if (new_state == OP_I) {
            p2 -= step;
        } else {
            p1 -= step;
        }
        if (new_state == state) {
            segment_length += step;
        } else {
            if (segment_length > 0) push(&l, state, (int)segment_length);
            segment_length = step;
            state = new_state;
        }
    } while (p1 > 0 && p2 > 0);
    int32_t off;
    if (strategy == SW_SOFTCLIP) {
        push(&l, state, (int)segment_length);
        if (p2 > 0) push(&l, OP_S, (int)p2);
        off = (int32_t)p1;
    } else if (strategy == SW_IGNORE) {
        push(&l, state, (int)(segment_length + p2));
        off = (int32_t)(p1 - p2);
    } else {
        push(&l, state, (int)segment_length);
        if (p1 > 0)
            push(&l, OP_D, (int)p1);
        else if (p2 > 0)
            push(&l, OP_I, (int)p2);
        off = 0;
    }
    free(sw), free(bt), free(best_gap_v), free(gap_size_v);
    if (l.overflow) return -2;
    for (int a = 0, b = l.n - 1; a < b; a++, b--) {
        const uint32_t t = ops[a];
        ops[a] = ops[b];
        ops[b] = t;
    }
    *n_ops = l.n;
    *offset = off;
    return 0;
}

/* Many pairs over the host threads (OpenMP; threads <= 0 uses every processor).  Pair p's ops go to
 * ops + ops_start[p], at most 2 * alt_len[p] + 4 of them.  Returns the first nonzero per-pair status, or 0. */
int sw_oracle_align_batch(int64_t n_pairs, const uint8_t *ref_plane, const int64_t *ref_off, const int32_t *ref_len,
                          const uint8_t *alt_plane, const int64_t *alt_off, const int32_t *alt_len,
                          const int32_t *params, int strategy, int shortcut, uint32_t *ops, const int64_t *ops_start,
                          int32_t *n_ops, int32_t *offset, int threads) {
    int status = 0;
#ifdef _OPENMP
    omp_set_num_threads(threads > 0 ? threads : omp_get_num_procs());
#else
    (void)threads;
#endif
#pragma omp parallel for schedule(dynamic, 16)
    for (int64_t p = 0; p < n_pairs; p++) {
        const int r = sw_oracle_align(ref_plane + ref_off[p], ref_len[p], alt_plane + alt_off[p], alt_len[p], params,
                                      strategy, shortcut, ops + ops_start[p], 2 * alt_len[p] + 4, n_ops + p,
                                      offset + p);
        if (r != 0) {
#pragma omp critical
            if (status == 0) status = r;
        }
    }
    return status;
}
