// Warp-level sorting networks on 64-bit keys held in registers.
#pragma once

#include <stdint.h>

namespace culof_gb300 {

__device__ __forceinline__ uint64_t shfl_xor_u64(uint64_t v, int mask) {
    return __shfl_xor_sync(0xffffffffu, v, mask);
}

// Bitonic sort of 32*E keys across a warp, ascending in element order
// e = j * 32 + lane (register j of lane `lane`). E must be a power of two.
template <int E>
__device__ __forceinline__ void warp_bitonic_sort(uint64_t (&v)[E]) {
    static_assert(E > 0 && (E & (E - 1)) == 0, "bitonic sort needs a power-of-two size");
    const int lane = threadIdx.x & 31;
    constexpr int N = 32 * E;
#pragma unroll
    for (int size = 2; size <= N; size <<= 1) {
#pragma unroll
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            if (stride >= 32) {
                const int rs = stride >> 5;  // register stride
#pragma unroll
                for (int j = 0; j < E; ++j) {
                    if ((j & rs) == 0) {
                        const int pj = j | rs;
                        const int e = j * 32 + lane;
                        const bool asc = (e & size) == 0;
                        const uint64_t a = v[j], b = v[pj];
                        const bool sw = asc ? (a > b) : (a < b);
                        v[j] = sw ? b : a;
                        v[pj] = sw ? a : b;
                    }
                }
            } else {
#pragma unroll
                for (int j = 0; j < E; ++j) {
                    const int e = j * 32 + lane;
                    const bool asc = (e & size) == 0;
                    const bool lower = (lane & stride) == 0;
                    const uint64_t o = shfl_xor_u64(v[j], stride);
                    const bool keep_min = (lower == asc);
                    v[j] = keep_min ? (o < v[j] ? o : v[j]) : (o > v[j] ? o : v[j]);
                }
            }
        }
    }
}

// After warp_bitonic_sort: flags the first copy of every distinct key that
// is not `sentinel`, returns the rank of each kept element among kept ones
// (or -1) and the number kept.
template <int E>
__device__ __forceinline__ int warp_unique_ranks(const uint64_t (&v)[E], uint64_t sentinel, int (&rank)[E]) {
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    int base = 0;
    uint64_t carry = ~v[0];  // previous element of element 0: anything different
#pragma unroll
    for (int j = 0; j < E; ++j) {
        uint64_t prev = __shfl_up_sync(0xffffffffu, v[j], 1);
        const uint64_t last_prev_reg = __shfl_sync(0xffffffffu, j > 0 ? v[j - 1] : carry, 31);
        if (lane == 0) prev = (j == 0) ? ~v[0] : last_prev_reg;
        const bool keep = v[j] != sentinel && v[j] != prev;
        const unsigned m = __ballot_sync(0xffffffffu, keep);
        rank[j] = keep ? base + __popc(m & lt_mask) : -1;
        base += __popc(m);
    }
    return base;
}

}  // namespace culof_gb300
