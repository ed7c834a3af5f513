// Pieces shared by the fused distance + filtered-select sweeps (fast.cu for
// small d, wide.cu for larger d): tiling constants, the filter threshold,
// packed FP32 helpers, mbarrier/TMA wrappers, and the per-row candidate
// lists with their compaction.
#pragma once

#include <stdint.h>

#include "common.cuh"
#include "warp_sort.cuh"

namespace culof_gb300 {
namespace sweep {

constexpr int kRT = 128;                   // rows per row tile
constexpr int kCT = 128;                   // columns per column tile
constexpr int kThreads = 256;              // 8 warps
constexpr int kWarps = kThreads / 32;
constexpr int kRowsPerWarp = kRT / kWarps;  // 16 rows owned by each warp
constexpr int kMaxK = 64;
constexpr int kQueueCap = 32 + 8 * 32;      // one rescoring chunk + one step's worth of candidates
constexpr unsigned kNoIndex = 0xFFFFFFFFu;
constexpr long long kSpinLimit = 1ll << 24;  // bounded mbarrier waits (~1-2 s with backoff)

// Column-tile visiting order of row tile T: T, T+1, T-1, T+2, T-2, ... mod nt
// (a permutation of 0..nt-1); sorted order is spatial, so nearby tiles first.
__device__ __forceinline__ int spiral_tile(int T, int q, int nt) {
    const int off = (q & 1) ? (q + 1) >> 1 : -(q >> 1);
    int t = (T + off) % nt;
    if (t < 0) t += nt;
    return t;
}

// Rigorous filter threshold. For a row a with float32 norm Na and any column
// b whose exact float32 direct-difference distance is <= kthD, the float32
// FMA chain e = fl(Nb + sum_f (-2 a_f) b_f) over dp terms satisfies
// e <= tau_from(...):
//   D <= kthD  =>  T = |a-b|^2 (real) <= kthD / (1 - (dp+2) u)
//   e_exact = T - |a|^2 + (Nb - |b|^2),  |a|^2 >= Na (1 - u),  Nb - |b|^2 <= u Nmax
//   |e - e_exact| <= gamma_{dp+1} (Nb + 2 sum|a_f b_f|) <= gamma (Nmax + 2 sqrt(Na Nmax)(1+u))
// plus 4u of slack for the double evaluation. Every term is evaluated in
// float32 rounded outward (divisions and products of the added terms up,
// the subtracted Na (1 - u) down, 1 + u taken as 1 + 2^-23), so the result
// bounds the formula from above; float32 instead of FP64 because this runs
// on every tightening of a row's k-th key and GB300's FP64 rate is low
// (the headline fit_predict: 7.47 -> 7.32 ms).
static __device__ float tau_from(uint64_t kth_key, float na, float nmax, int dp) {
    if (kth_key == kKeyMax) return __int_as_float(0x7f800000);
    const float D = __uint_as_float(key_bits(kth_key));
    const float u = 5.9604644775390625e-08f;             // 2^-24
    const float tm = __fdiv_ru(D, 1.0f - (dp + 2) * u);  // both operands exact
    const float gam = __fdiv_ru((dp + 1) * u, 1.0f - (dp + 1) * u);
    const float a_lo = __fmul_rd(na, 1.0f - u);
    const float root = __fmul_ru(__fmul_ru(2.0f, __fsqrt_ru(__fmul_ru(na, nmax))), 1.00000011920928955f);
    float t = __fsub_ru(tm, a_lo);
    t = __fadd_ru(t, __fmul_ru(u, nmax));
    t = __fadd_ru(t, __fmul_ru(gam, __fadd_ru(nmax, root)));
    t = __fadd_ru(t, __fmul_ru(4.0f * u, __fadd_ru(__fadd_ru(tm, na), nmax)));
    return __fadd_ru(t, 1e-30f);
}

__device__ __forceinline__ uint64_t fma2(uint64_t a, uint64_t b, uint64_t c) {
    uint64_t d;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(a), "l"(b), "l"(c));
    return d;
}
__device__ __forceinline__ uint64_t dup2(float x) {
    const uint64_t u = __float_as_uint(x);
    return u | (u << 32);
}
__device__ __forceinline__ float lo_f(uint64_t v) { return __uint_as_float(static_cast<uint32_t>(v)); }
__device__ __forceinline__ float hi_f(uint64_t v) { return __uint_as_float(static_cast<uint32_t>(v >> 32)); }

// ---- mbarrier / TMA ---------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, unsigned parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
// Bounded wait: false if the phase never completes (the caller reports it).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, long long limit = kSpinLimit) {
    for (long long it = 0; it < limit; ++it) {
        if (mbar_try_wait(bar, parity)) return true;
        if (it > 64) __nanosleep(64);
    }
    return false;
}
// Warp-uniform bounded wait: every lane polls, and the warp leaves the loop
// together (all lanes saw the phase complete, or all gave up), so no lane
// can run ahead into warp-synchronous code alone.
__device__ __forceinline__ bool mbar_wait_warp(uint64_t* bar, unsigned parity) {
    for (long long it = 0; it < kSpinLimit; ++it) {
        if (__all_sync(0xffffffffu, mbar_try_wait(bar, parity))) return true;
        if (it > 64) __nanosleep(64);
    }
    return false;
}
// Plain arrive (no transaction bytes): completes a phase that expects no copy.
__device__ __forceinline__ void mbar_arrive_plain(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ void tma_load_1d(void* smem_dst, const void* gmem_src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_u32(smem_dst)),
        "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// ---- per-row candidate lists ---------------------------------------------------
// list[r][0..cnt) holds keys (exact distance bits, original index) that beat
// the row's k-th key at the time they were added; kth[r] only ever decreases
// and tau[r] is its filter threshold. Rows are owned by warps (16 each), so
// only the owning warp touches a row's list.
template <int M>
struct RowLists {
    uint64_t list[kRT][M];
    uint64_t kth[kRT];
    float tau[kRT];
    float row_norm[kRT];
    int cnt[kRT];
    int sorted[kRT];  // list[r][0..sorted) is sorted and unique (the last compaction's result)
};

// Compact row r's list (whole warp): sort, drop duplicates, keep the k
// smallest; tighten the row's k-th key (only downwards) and its threshold.
template <int M>
__device__ void compact_row(RowLists<M>& L, int r, int k, float nmax, int dp) {
    if constexpr (M <= 64) {
        // nothing added since the last compaction: the list is already its
        // sorted k best; at most 32 added: sort those and merge them with
        // the sorted prefix (keys are unique: every pair is offered once)
        const int c = min(L.cnt[r], M), s = L.sorted[r];
        if (s >= 0 && s == c) return;
        if (s >= 0 && s < c && c - s <= 32) {
            uint64_t kk;
            const int kept =
                merge_sorted_prefix<1>(L.list[r], s, c, k, k - 1, [](uint64_t) { return kKeyMax; }, &kk);
            if ((threadIdx.x & 31) == 0) {
                L.cnt[r] = kept;
                L.sorted[r] = kept;
                if (kk != kKeyMax && kk < L.kth[r]) {
                    L.kth[r] = kk;
                    L.tau[r] = tau_from(kk, L.row_norm[r], nmax, dp);
                }
            }
            __syncwarp();
            return;
        }
    }
    if constexpr (M > 64) {
        // fast form for lists the full network sorts as 128 keys: sort only
        // the entries added since the last compaction (at most 64) and merge
        // them with its sorted result
        const int c = min(L.cnt[r], M), s = L.sorted[r];
        if (s >= 0 && s <= c && s <= 128 && c - s <= 64) {
            uint64_t kk;
            const int kept = merge_sorted_prefix(L.list[r], s, c, k, k - 1, [](uint64_t) { return kKeyMax; }, &kk);
            if ((threadIdx.x & 31) == 0) {
                L.cnt[r] = kept;
                L.sorted[r] = kept;
                if (kk != kKeyMax && kk < L.kth[r]) {
                    L.kth[r] = kk;
                    L.tau[r] = tau_from(kk, L.row_norm[r], nmax, dp);
                }
            }
            __syncwarp();
            return;
        }
    }
    // the bitonic network needs a power of two: ceil(M / 32) registers per
    // lane, padded up to one (with kKeyMax)
    constexpr int R = (M + 31) / 32;
    constexpr int E = R <= 1 ? 1 : R <= 2 ? 2 : R <= 4 ? 4 : 8;
    static_assert(32 * E >= M, "the sort covers the whole list");
    static_assert(M % 8 == 0 && M <= 256, "list capacity");
    const int lane = threadIdx.x & 31;
    const int c = min(L.cnt[r], M);
    uint64_t v[E];
#pragma unroll
    for (int j = 0; j < E; ++j) {
        const int e = j * 32 + lane;
        v[j] = e < c ? L.list[r][e] : kKeyMax;
    }
    warp_bitonic_sort<E>(v);
    int rank[E];
    const int uniq = warp_unique_ranks<E>(v, kKeyMax, rank);
    __syncwarp();
    uint64_t kth_new = kKeyMax;
#pragma unroll
    for (int j = 0; j < E; ++j) {
        if (rank[j] >= 0 && rank[j] < k) L.list[r][rank[j]] = v[j];
        if (rank[j] == k - 1) kth_new = v[j];
    }
    const unsigned m = __ballot_sync(0xffffffffu, kth_new != kKeyMax);
    const uint64_t kk = __shfl_sync(0xffffffffu, kth_new, m ? __ffs(m) - 1 : 0);
    __syncwarp();
    if (lane == 0) {
        L.cnt[r] = min(uniq, k);
        L.sorted[r] = min(uniq, k);
        if (m && kk < L.kth[r]) {
            L.kth[r] = kk;
            L.tau[r] = tau_from(kk, L.row_norm[r], nmax, dp);
        }
    }
    __syncwarp();
}

// Compact every row of this warp whose list has less than 32 free slots
// (so the next chunk of 32 appends cannot overflow). True if any was.
template <int M>
__device__ bool compact_full_rows(RowLists<M>& L, int k, float nmax, int dp) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int row0 = warp * kRowsPerWarp;
    unsigned full = __ballot_sync(0xffffffffu, lane < kRowsPerWarp && L.cnt[row0 + lane] > M - 32);
    const bool any = full != 0;
    while (full) {
        compact_row<M>(L, row0 + __ffs(full) - 1, k, nmax, dp);
        full &= full - 1;
    }
    return any;
}

// Warp-ordered append of this lane's `count` candidate codes (from `codes`)
// to the warp queue at qc; returns the new count.
__device__ __forceinline__ int warp_prefix_offset(int count, int& total) {
    const int lane = threadIdx.x & 31;
    int off = count;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, off, o);
        if (lane >= o) off += y;
    }
    total = __shfl_sync(0xffffffffu, off, 31);
    return off - count;
}

}  // namespace sweep
}  // namespace culof_gb300
