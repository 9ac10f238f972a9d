/*
 * oracle_grad.c -- FP64 forward and forward-backward gradient oracle for the
 * continuous-parameter PairHMM used by gap-penalty calibration.
 *
 * TEST INFRASTRUCTURE ONLY (see pairhmm_oracle.c).  Never linked by the product.
 *
 * Model.  The recurrence is LoglessPairHMM's (LoglessPairHMM.java:47-67) with the
 * per-row transitions written in the continuous form of PairHMMModel.qualToTransProbs
 * (PairHMMModel.java:107-117): with g = gap-open log10-probability and c = gap-continuation
 * log10-probability of read position i-1 (row i, PairHMMModel.java:169-171),
 *     MI = MD = 10^g,  MM = 1 - 2*10^g,  II = DD = 10^c,  IM = 1 - 10^c.
 * MM = 1 - 2*10^g is the exact value that the Jacobian-table matchToMatch entry
 * (PairHMMModel.java:86-94) approximates for equal insertion and deletion penalties.
 * Priors come from base qualities exactly as LoglessPairHMM.initializePriors (:79-93).
 *
 * The gradient is computed by the adjoint (backward) recurrence over full FP64
 * matrices; it is the reference gradient that the GPU backward kernel is checked against,
 * alongside central finite differences of oracle_cont_forward.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>

double oracle_qual_to_error_prob(int q);
double oracle_qual_to_prob(int q);

static int og_is_match(uint8_t x, uint8_t y) { return x == y || x == (uint8_t)'N' || y == (uint8_t)'N'; }

typedef struct {
    double a, b, e, f, h, k; /* MM, IM, MI, II, MD, DD */
} og_trans;

static void og_row_trans(double g, double c, og_trans *t) {
    const double pg = pow(10.0, g), pc = pow(10.0, c);
    t->a = 1.0 - 2.0 * pg;
    t->e = pg;
    t->h = pg;
    t->b = 1.0 - pc;
    t->f = pc;
    t->k = pc;
}

/* log10 L of one pair under per-row continuous parameters g[0..R-1], c[0..R-1]. */
double oracle_cont_forward(const uint8_t *hap, int H, const uint8_t *rb, const uint8_t *q, const double *g,
                           const double *c, int R) {
    const double init_cond = ldexp(1.0, 1020);
    double *buf = (double *)calloc((size_t)6 * (size_t)(H + 1), sizeof(double));
    double *Mp = buf, *Ip = buf + (H + 1), *Dp = buf + 2 * (H + 1);
    double *Mc = buf + 3 * (H + 1), *Ic = buf + 4 * (H + 1), *Dc = buf + 5 * (H + 1);
    for (int j = 0; j <= H; j++) Dp[j] = init_cond / (double)H;
    for (int i = 1; i <= R; i++) {
        og_trans t;
        og_row_trans(g[i - 1], c[i - 1], &t);
        const double pm = oracle_qual_to_prob(q[i - 1]);
        const double pe = oracle_qual_to_error_prob(q[i - 1]) / 3.0;
        Mc[0] = Ic[0] = Dc[0] = 0.0;
        for (int j = 1; j <= H; j++) {
            const double pr = og_is_match(rb[i - 1], hap[j - 1]) ? pm : pe;
            Mc[j] = pr * (Mp[j - 1] * t.a + Ip[j - 1] * t.b + Dp[j - 1] * t.b);
            Ic[j] = Mp[j] * t.e + Ip[j] * t.f;
            Dc[j] = Mc[j - 1] * t.h + Dc[j - 1] * t.k;
        }
        double *s;
        s = Mp; Mp = Mc; Mc = s;
        s = Ip; Ip = Ic; Ic = s;
        s = Dp; Dp = Dc; Dc = s;
    }
    double sum = 0.0;
    for (int j = 1; j <= H && R > 0; j++) sum += Mp[j] + Ip[j];
    free(buf);
    return log10(sum) - log10(init_cond);
}

/*
 * log10 L and its gradient with respect to g[i] and c[i] (i = 0..R-1), by the adjoint
 * recurrence.  dg, dc receive d log10 L / d g_i and d log10 L / d c_i.
 */
double oracle_cont_grad(const uint8_t *hap, int H, const uint8_t *rb, const uint8_t *q, const double *g,
                        const double *c, int R, double *dg, double *dc) {
    const double init_cond = ldexp(1.0, 1020);
    const size_t W = (size_t)(H + 1), N = (size_t)(R + 1) * W;
    double *M = (double *)calloc(N, sizeof(double));
    double *I = (double *)calloc(N, sizeof(double));
    double *D = (double *)calloc(N, sizeof(double));
    double *P = (double *)calloc(N, sizeof(double));
    og_trans *T = (og_trans *)calloc((size_t)R + 2, sizeof(og_trans));
    for (int j = 0; j <= H; j++) D[j] = init_cond / (double)H;
    for (int i = 1; i <= R; i++) {
        og_row_trans(g[i - 1], c[i - 1], &T[i]);
        const double pm = oracle_qual_to_prob(q[i - 1]);
        const double pe = oracle_qual_to_error_prob(q[i - 1]) / 3.0;
        for (int j = 1; j <= H; j++) {
            const size_t x = (size_t)i * W + (size_t)j;
            P[x] = og_is_match(rb[i - 1], hap[j - 1]) ? pm : pe;
            M[x] = P[x] * (M[x - W - 1] * T[i].a + I[x - W - 1] * T[i].b + D[x - W - 1] * T[i].b);
            I[x] = M[x - W] * T[i].e + I[x - W] * T[i].f;
            D[x] = M[x - 1] * T[i].h + D[x - 1] * T[i].k;
        }
    }
    double L = 0.0;
    for (int j = 1; j <= H; j++) L += M[(size_t)R * W + (size_t)j] + I[(size_t)R * W + (size_t)j];

    /* adjoints, reusing three fresh matrices */
    double *bM = (double *)calloc(N, sizeof(double));
    double *bI = (double *)calloc(N, sizeof(double));
    double *bD = (double *)calloc(N, sizeof(double));
    for (int i = R; i >= 1; i--) {
        for (int j = H; j >= 1; j--) {
            const size_t x = (size_t)i * W + (size_t)j;
            double vm = (i == R) ? 1.0 : 0.0, vi = vm, vd = 0.0;
            if (i < R && j < H) {
                const double t = bM[x + W + 1] * P[x + W + 1];
                vm += t * T[i + 1].a;
                vi += t * T[i + 1].b;
                vd += t * T[i + 1].b;
            }
            if (i < R) {
                vm += bI[x + W] * T[i + 1].e;
                vi += bI[x + W] * T[i + 1].f;
            }
            if (j < H) {
                vm += bD[x + 1] * T[i].h;
                vd += bD[x + 1] * T[i].k;
            }
            bM[x] = vm;
            bI[x] = vi;
            bD[x] = vd;
        }
    }
    const double ln10 = log(10.0);
    for (int i = 1; i <= R; i++) {
        double da = 0, db = 0, de = 0, df = 0, dh = 0, dk = 0;
        for (int j = 1; j <= H; j++) {
            const size_t x = (size_t)i * W + (size_t)j;
            da += bM[x] * P[x] * M[x - W - 1];
            db += bM[x] * P[x] * (I[x - W - 1] + D[x - W - 1]);
            de += bI[x] * M[x - W];
            df += bI[x] * I[x - W];
            dh += bD[x] * M[x - 1];
            dk += bD[x] * D[x - 1];
        }
        const double pg = pow(10.0, g[i - 1]), pc = pow(10.0, c[i - 1]);
        /* d/dg: e = h = 10^g, a = 1 - 2*10^g ; d/dc: f = k = 10^c, b = 1 - 10^c */
        const double dLdg = ln10 * pg * (de + dh - 2.0 * da);
        const double dLdc = ln10 * pc * (df + dk - db);
        dg[i - 1] = dLdg / (L * ln10);
        dc[i - 1] = dLdc / (L * ln10);
    }
    free(M); free(I); free(D); free(P); free(T); free(bM); free(bI); free(bD);
    return log10(L) - log10(init_cond);
}
