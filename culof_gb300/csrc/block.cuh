// Block-level building blocks (warp-shuffle scans), written for blocks whose
// size is a multiple of 32 and at most 1024.
#pragma once

#include <cuda_runtime.h>

namespace culof_gb300 {

__device__ __forceinline__ int warp_inclusive_scan(int v) {
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
    }
    return v;
}

// Exclusive prefix sum over the block in thread order; `total` receives the
// block-wide sum. `warp_sums` is shared scratch of blockDim.x / 32 ints.
// Contains __syncthreads(): every thread of the block must call it.
__device__ __forceinline__ int block_exclusive_scan(int v, int* warp_sums, int& total) {
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int nwarps = blockDim.x >> 5;
    const int incl = warp_inclusive_scan(v);
    if (lane == 31) warp_sums[warp] = incl;
    __syncthreads();
    if (warp == 0) {
        int w = lane < nwarps ? warp_sums[lane] : 0;
        w = warp_inclusive_scan(w);
        if (lane < nwarps) warp_sums[lane] = w;
    }
    __syncthreads();
    const int base = warp > 0 ? warp_sums[warp - 1] : 0;
    total = warp_sums[nwarps - 1];
    __syncthreads();  // warp_sums may be reused by the caller right away
    return base + incl - v;
}

}  // namespace culof_gb300
