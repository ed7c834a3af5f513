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

// The 32 smallest of two ascending 32-key runs a and b (one key per lane,
// element = lane), ascending: the elementwise minimum of a and reversed b is
// a bitonic sequence holding them, and five half-cleaner steps sort it.
__device__ __forceinline__ uint64_t warp_merge_lowest32(uint64_t a, uint64_t b) {
    const int lane = threadIdx.x & 31;
    const uint64_t rb = __shfl_sync(0xffffffffu, b, 31 - lane);
    uint64_t c = a < rb ? a : rb;
#pragma unroll
    for (int st = 16; st > 0; st >>= 1) {
        const uint64_t o = shfl_xor_u64(c, st);
        c = (lane & st) == 0 ? (o < c ? o : c) : (o > c ? o : c);
    }
    return c;
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

// Number of entries of the ascending array a[0..len) below x (binary search).
__device__ __forceinline__ int count_below(const uint64_t* a, int len, uint64_t x) {
    int lo = 0, hi = len;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < x) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Merge compaction of a list whose first s entries are sorted ascending and
// whose entries s..c are new and unsorted (whole warp; keys unique; requires
// s <= 128 and c - s <= 32 E). The new entries are sorted (a 32 E-key bitonic
// network) and written back behind the prefix; every element's merged rank
// is its index in its own run plus the number of smaller keys in the other
// run (a binary search). Once the key of merged rank sel_rank is known
// (kKeyMax if there is none), bound_fn(that key) gives an inclusive upper
// bound: the merged keys <= bound, at most keep_max of them, are written to
// lst[0..) in ascending order. Returns how many were kept; *sel receives the
// selected key.
template <int E = 2, typename BoundFn>
__device__ __forceinline__ int merge_sorted_prefix(uint64_t* lst, int s, int c, int keep_max, int sel_rank,
                                                   BoundFn bound_fn, uint64_t* sel) {
    const int lane = threadIdx.x & 31;
    const int u = c - s;
    uint64_t v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const int e = j * 32 + lane;
        v[j] = e < u ? lst[s + e] : ~0ull;
    }
    warp_bitonic_sort<E>(v);
    __syncwarp();
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const int e = j * 32 + lane;
        if (e < u) lst[s + e] = v[j];
    }
    __syncwarp();
    uint64_t p[4];
    int pr[4], vr[E];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const int e = j * 32 + lane;
        p[j] = e < s ? lst[e] : ~0ull;
        pr[j] = e < s ? e + count_below(lst + s, u, p[j]) : -1;
    }
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const int e = j * 32 + lane;
        vr[j] = e < u ? e + count_below(lst, s, v[j]) : -1;
    }
    uint64_t mine = ~0ull;
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (pr[j] == sel_rank) mine = p[j];
#pragma unroll
    for (int j = 0; j < E; ++j)
        if (vr[j] == sel_rank) mine = v[j];
    const unsigned m = __ballot_sync(0xffffffffu, mine != ~0ull);
    const uint64_t picked = m ? __shfl_sync(0xffffffffu, mine, __ffs(m) - 1) : ~0ull;
    *sel = picked;
    const uint64_t bound = bound_fn(picked);
    // merged keys <= bound form a prefix of the merged order
    int below = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) below += __popc(__ballot_sync(0xffffffffu, pr[j] >= 0 && p[j] <= bound));
#pragma unroll
    for (int j = 0; j < E; ++j) below += __popc(__ballot_sync(0xffffffffu, vr[j] >= 0 && v[j] <= bound));
    const int keep = below < keep_max ? below : keep_max;
    __syncwarp();
#pragma unroll
    for (int j = 0; j < 4; ++j)
        if (pr[j] >= 0 && pr[j] < keep) lst[pr[j]] = p[j];
#pragma unroll
    for (int j = 0; j < E; ++j)
        if (vr[j] >= 0 && vr[j] < keep) lst[vr[j]] = v[j];
    __syncwarp();
    return keep;
}

}  // namespace culof_gb300
