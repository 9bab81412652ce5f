// Internal declarations shared by the host and device translation units.
#pragma once
#include <cstdint>

namespace btc {

// U(lo, hi) value for factor (mode, row, col) from a counter-based generator.
double init_uniform(uint64_t seed, int mode, int64_t row, int col, double lo, double hi);

}  // namespace btc
