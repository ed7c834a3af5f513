// Host entry points of the tensor-core stages (tc.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace culof_gb300 {
namespace tc {

// G (rows_a x rows_b, row-major f32) = A B^T for row-major bf16 A, B with K = 128.
void bf16_gram(const void* A, int64_t rows_a, const void* B, int64_t rows_b, int K, float* G, int* status,
               cudaStream_t s);

}  // namespace tc
}  // namespace culof_gb300
