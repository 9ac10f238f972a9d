// str_analyzer.cpp -- short-tandem-repeat (period, repeat count) of every read position, as the DRAGstr
// gap-penalty model reads it (src/main/java/org/broadinstitute/hellbender/utils/pairhmm/
// DragstrReadSTRAnalyzer.java:11-46, :110-136, :148-285).
//
// For position i and period p, the repeat count is the largest tandem run (in units of p, counted up-
// and downstream) of any p-mer that contains i, or of the p-mer starting at i+1.  A unit starting at 0
// loses one repeat (not below 1) for positions i < p-1 (DRAGEN's convention, reproduced by the reference).
// The most repeated period wins, ties going to the shorter period.  Every p-mer's run is found with two
// passes over "unit at x equals unit at x+p" flags, O(n) per period.
#include <algorithm>
#include <cstdint>
#include <vector>

#include "../../include/ghmm_calib.h"
#include "str_analyzer.h"

namespace ghmm {

void str_repeats_for_period(const uint8_t *s, int n, int p, int32_t *out) {
    if (p > n) {
        std::fill(out, out + n, 0);
        return;
    }
    const int nu = n - p + 1;  // unit starts 0 .. n-p
    // eqrun[y]: number of consecutive y' >= y with s[y'] == s[y'+p]
    std::vector<int> eqrun((size_t)n + 1, 0);
    for (int y = n - p - 1; y >= 0; --y) eqrun[(size_t)y] = (s[y] == s[y + p]) ? eqrun[(size_t)y + 1] + 1 : 0;
    // next[x]: unit at x equals unit at x+p (both inside the sequence)
    auto next_eq = [&](int x) { return x + 2 * p <= n && eqrun[(size_t)x] >= p; };
    std::vector<int> fwd((size_t)nu, 0), bwd((size_t)nu, 0), run((size_t)nu, 0);
    for (int x = nu - 1; x >= 0; --x) fwd[(size_t)x] = next_eq(x) ? 1 + fwd[(size_t)x + (size_t)p] : 0;
    for (int x = 0; x < nu; ++x) bwd[(size_t)x] = (x >= p && next_eq(x - p)) ? 1 + bwd[(size_t)(x - p)] : 0;
    for (int x = 0; x < nu; ++x) run[(size_t)x] = 1 + fwd[(size_t)x] + bwd[(size_t)x];
    for (int i = 0; i < n; ++i) {
        const int lo = std::max(0, i - p + 1), hi = std::min(i + 1, nu - 1);
        int best = 0;
        for (int x = lo; x <= hi; ++x) {
            int c = run[(size_t)x];
            if (x == 0 && i < p - 1) c = std::max(1, c - 1);
            best = std::max(best, c);
        }
        out[i] = best;
    }
}

void str_analyze(const uint8_t *s, int n, int max_period, int32_t *best_period, int32_t *best_repeats,
                 int32_t *all_repeats) {
    std::vector<int32_t> rep((size_t)n);
    for (int i = 0; i < n; ++i) {
        best_period[i] = 1;
        best_repeats[i] = 0;
    }
    for (int p = 1; p <= max_period; ++p) {
        str_repeats_for_period(s, n, p, rep.data());
        for (int i = 0; i < n; ++i) {
            if (all_repeats) all_repeats[(size_t)(p - 1) * (size_t)n + (size_t)i] = rep[(size_t)i];
            if (p == 1 || rep[(size_t)i] > best_repeats[i]) {
                best_repeats[i] = rep[(size_t)i];
                best_period[i] = p;
            }
        }
    }
}

}  // namespace ghmm

extern "C" int ghmm_str_analyze(const uint8_t *bases, int32_t n, int32_t max_period, int32_t *best_period,
                                int32_t *best_repeats, int32_t *all_repeats) {
    if (n < 0 || max_period < 1 || (n > 0 && (!bases || !best_period || !best_repeats))) return 1;
    if (n == 0) return 0;
    ghmm::str_analyze(bases, n, max_period, best_period, best_repeats, all_repeats);
    return 0;
}
