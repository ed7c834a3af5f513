// Fused distance + filtered exact select (the fast k-NN path).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace culof_gb300 {

// True when the fast path handles (n, d, k).
bool fast_path_supported(int64_t n, int d, int k);

// The wide-point variant (8 < d <= 128), wide.cu.
int wide_dims_padded(int d);
size_t wide_tiles_floats(int d, int nt);
void wide_build_tiles(const float* xc, const float* norms, int64_t n, int d, const unsigned* perm, int nt,
                      float* tiles, cudaStream_t s);
void wide_seed(const float* tiles, int nt, int d, int k, uint64_t* seed_keys, unsigned long long* kth_shared,
               cudaStream_t s);
void wide_sweep(const float* tiles, int nt, int nsplit, int d, int k, const unsigned* maxn,
                unsigned long long* kth_shared, uint64_t* partial, cudaStream_t s);

}  // namespace culof_gb300
