// str_analyzer.h -- DRAGstr read STR analysis (see str_analyzer.cpp).
#pragma once

#include <cstdint>

namespace ghmm {

// Repeat count at every position for one period p (out[n]).
void str_repeats_for_period(const uint8_t *s, int n, int p, int32_t *out);
// Most repeated period and its repeat count at every position; all_repeats (optional) is
// [max_period][n] with the count of every period.
void str_analyze(const uint8_t *s, int n, int max_period, int32_t *best_period, int32_t *best_repeats,
                 int32_t *all_repeats);

}  // namespace ghmm
