#include "engine.cuh"
#include "fast.cuh"

namespace culof_gb300 {

bool fast_path_supported(int64_t, int, int) { return false; }

void Engine::knn_fast(const float*, const float*, int64_t, int, int, int32_t*, float*, float*) {
    throw Error(kInternal, "fast path not built");
}

}  // namespace culof_gb300
