// Fused distance + filtered exact select (the fast k-NN path).
#pragma once

#include <stdint.h>

namespace culof_gb300 {

// True when the fast path handles (n, d, k).
bool fast_path_supported(int64_t n, int d, int k);

}  // namespace culof_gb300
