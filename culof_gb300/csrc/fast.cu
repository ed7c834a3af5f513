// The fast exact k-NN path: fused distance + filtered exact select.
//
// Replaces the reference's hot loop (pipeline.cu:175-195: cuBLAS SGEMM of a
// rows x n Gram tile to HBM, then knn_select_kernel's four sweeps of it,
// knn.cu:119-232, ~24 B of HBM traffic per pair) with one evaluation per
// pair that never leaves the SM:
//
//  1. spatial order: a 32-bit Morton key of the centred coordinates, sorted
//     with a stable LSD radix sort; tiles of 128 consecutive sorted points
//     are spatially compact.
//  2. seed: per row, the exact k best over its own tile and the four nearest
//     tiles in Morton order (T+-1, T+-2), by warp bitonic sorts and merges.
//     Its k-th key K bounds the row's true k-th key; the sweep covers every
//     later tile.
//  3. sweep: each CTA owns 128 rows and streams column tiles (TMA bulk
//     copies into shared memory, nearest tiles first); each warp owns 16 of
//     the rows (4 per lane, in registers as -2a). For every pair it
//     evaluates e = |b|^2 - 2 a.b with packed fma.rn.f32x2 (two columns per
//     instruction) and compares with a per-row threshold tau, a rigorous
//     float32 error bound over the row's current k-th key K, so every column
//     that can still enter the k best passes. Passing pairs are queued per
//     warp and rescored 32 at a time (exact distance, the oracle's formula);
//     keys that beat K join the row's list in shared memory, and filling
//     lists are compacted (bitonic sort, dedup, keep k), tightening K and
//     tau. K is shared across the column splits of a row tile through
//     global memory (atomicMin), so later splits start from earlier ones'.
//  4. merge: the seed list and the S column-split lists give the k best
//     keys; slots are written in the reference's order (keys below the k-th
//     by ascending index, then the ties, knn.cu:190-224).
//
// Exactness: the selection key is (exact float32 distance bits, original
// index), identical to the general path and the oracle; the filter only
// decides which pairs get an exact evaluation, and its bound is proven
// conservative (tau_from below).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>

#include "common.cuh"
#include "engine.cuh"
#include "fast.cuh"
#include "sweep_common.cuh"
#include "warp_sort.cuh"

namespace culof_gb300 {

namespace {

using namespace sweep;

constexpr int kPairs = kCT / 2;
constexpr int kRowsPerLane = 4;
constexpr int kStages = 5;     // column tiles in flight
constexpr int kSeedWindow = 5;  // tiles of the seed: T, T+1, T-1, T+2, T-2
constexpr int kMaxDP = 8;      // the small-d sweep; wider points take wide.cu's
constexpr int kMaxWideD = 128;
constexpr int kMortonDims = 8;  // Morton key over (up to) the 8 widest dimensions

// ---------------------------------------------------------------- layout
// Column tile t (kCT consecutive sorted points) in global memory and, when
// staged, in shared memory:
//   coords: kPairs pair records of pair_stride(DP) floats; pair p holds
//           columns (2p, 2p+1) interleaved per dimension,
//           [b_2p[0], b_2p+1[0], b_2p[1], b_2p+1[1], ...], then padding so
//           that eight pair records read by one warp hit distinct banks
//   norms : kCT floats (NaN for padding columns)
//   index : kCT uint32 original indices (kNoIndex for padding)
//   box   : per-dimension minimum and maximum over the tile's valid points
// The CTA's own rows are the columns of its own tile.
__host__ __device__ constexpr int pair_stride(int dp) { return ((2 * dp / 4) % 2 == 1) ? 2 * dp : 2 * dp + 4; }
__host__ __device__ constexpr int tile_norms_off(int dp) { return kPairs * pair_stride(dp); }
__host__ __device__ constexpr int tile_index_off(int dp) { return tile_norms_off(dp) + kCT; }
// bounding box of the tile's valid points: lo[DP], hi[DP] (padding dims 0)
__host__ __device__ constexpr int tile_box_off(int dp) { return tile_index_off(dp) + kCT; }
__host__ __device__ constexpr int tile_floats(int dp) { return tile_box_off(dp) + 2 * dp; }
__host__ __device__ constexpr int tile_bytes(int dp) { return tile_floats(dp) * 4; }

// Coordinate f of column c within a tile.
template <int DP>
__device__ __forceinline__ float tile_coord(const float* tile, int c, int f) {
    return tile[(c >> 1) * pair_stride(DP) + 2 * f + (c & 1)];
}

__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
// The next float above t (t itself for +-inf): x <= t  <=>  x < tau_above(t).
__device__ __forceinline__ float tau_above(float t) {
    return (isinf(t)) ? t : nextafterf(t, __int_as_float(0x7f800000));
}

// ---------------------------------------------------------------- spatial order

__device__ __forceinline__ unsigned flip_float(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unflip_float(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// Per dimension f: mm[2f] = min key, mm[2f+1] = max key (flipped floats).
// One coalesced pass over the n x d values: each thread stays on one
// dimension (the block's active threads and its stride are multiples of d),
// reduces in shared memory, and one thread per dimension and block updates
// the global words. Requires d <= kMaxMinmaxDims.
constexpr int kMaxMinmaxDims = 256;
__global__ void minmax_kernel(const float* __restrict__ xc, int64_t n, int d, unsigned* __restrict__ mm) {
    __shared__ unsigned slo[kMaxMinmaxDims], shi[kMaxMinmaxDims];
    for (int f = threadIdx.x; f < d; f += blockDim.x) {
        slo[f] = 0xFFFFFFFFu;
        shi[f] = 0u;
    }
    __syncthreads();
    const int per = static_cast<int>(blockDim.x) / d * d;  // active threads
    if (static_cast<int>(threadIdx.x) < per) {
        const int f = static_cast<int>(threadIdx.x) % d;
        unsigned lo = 0xFFFFFFFFu, hi = 0u;
        const int64_t total = n * d;
        for (int64_t t = static_cast<int64_t>(blockIdx.x) * per + threadIdx.x; t < total;
             t += static_cast<int64_t>(gridDim.x) * per) {
            const unsigned k = flip_float(xc[t]);
            lo = min(lo, k);
            hi = max(hi, k);
        }
        atomicMin(&slo[f], lo);
        atomicMax(&shi[f], hi);
    }
    __syncthreads();
    for (int f = threadIdx.x; f < d; f += blockDim.x) {
        atomicMin(&mm[2 * f], slo[f]);
        atomicMax(&mm[2 * f + 1], shi[f]);
    }
}

__global__ void minmax_init_kernel(unsigned* mm, int d) {
    for (int f = threadIdx.x; f < d; f += blockDim.x) {
        mm[2 * f] = 0xFFFFFFFFu;
        mm[2 * f + 1] = 0u;
    }
}

// The (up to) kMortonDims dimensions with the widest range, widest first
// (ties by index); one thread.
__global__ void select_dims_kernel(const unsigned* __restrict__ mm, int d, int* __restrict__ dims) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const int m = d < kMortonDims ? d : kMortonDims;
    for (int j = 0; j < m; ++j) {
        int best = -1;
        float best_span = -1.0f;
        for (int f = 0; f < d; ++f) {
            bool taken = false;
            for (int q = 0; q < j; ++q) taken |= dims[q] == f;
            if (taken) continue;
            const float span = unflip_float(mm[2 * f + 1]) - unflip_float(mm[2 * f]);
            if (span > best_span) {
                best_span = span;
                best = f;
            }
        }
        dims[j] = best;
    }
}

// 32-bit Morton key: 32/m bits for each of the m selected dimensions,
// interleaved from the most significant bit, over the bounding box of the
// centred data.
__global__ void morton_kernel(const float* __restrict__ xc, int64_t n, int d, const unsigned* __restrict__ mm,
                              const int* __restrict__ dims, unsigned* __restrict__ keys, unsigned* __restrict__ vals) {
    const int md = d < kMortonDims ? d : kMortonDims;
    const int bits = (32 / md) < 30 ? (32 / md) : 30;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        unsigned q[kMortonDims];
        for (int j = 0; j < md; ++j) {
            const int f = dims[j];
            const float lo = unflip_float(mm[2 * f]), hi = unflip_float(mm[2 * f + 1]);
            const float span = hi - lo;
            float t = span > 0.0f ? (xc[i * d + f] - lo) / span : 0.0f;
            t = fminf(fmaxf(t, 0.0f), 1.0f);
            const float scale = static_cast<float>((1u << bits) - 1u);
            q[j] = static_cast<unsigned>(t * scale + 0.5f);
        }
        unsigned key = 0u;
        for (int b = bits - 1; b >= 0; --b)
            for (int j = 0; j < md; ++j) key = (key << 1) | ((q[j] >> b) & 1u);
        keys[i] = key;
        vals[i] = static_cast<unsigned>(i);
    }
}

// ---- stable LSD radix sort, 8-bit digits, 2048 items per block -------------
constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr int kSortTile = kSortThreads * kSortItems;

__global__ void sort_upsweep_kernel(const unsigned* __restrict__ keys, int64_t n, int shift,
                                    unsigned* __restrict__ counts, int nblocks) {
    __shared__ unsigned hist[256];
    hist[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kSortTile;
    for (int it = 0; it < kSortItems; ++it) {
        const int64_t i = base + static_cast<int64_t>(it) * kSortThreads + threadIdx.x;
        if (i < n) atomicAdd(&hist[(keys[i] >> shift) & 0xFF], 1u);
    }
    __syncthreads();
    counts[static_cast<int64_t>(threadIdx.x) * nblocks + blockIdx.x] = hist[threadIdx.x];
}

// Exclusive scan of counts[256 * nblocks] in digit-major order (one block):
// each thread scans kScanItems consecutive counts per step, the block scans
// the threads' totals.
constexpr int kScanItems = 8;
__global__ void sort_scan_kernel(unsigned* __restrict__ counts, int64_t len) {
    __shared__ unsigned warp_tot[32];
    __shared__ unsigned carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t step = static_cast<int64_t>(blockDim.x) * kScanItems;
    for (int64_t base = 0; base < len; base += step) {
        const int64_t i0 = base + static_cast<int64_t>(threadIdx.x) * kScanItems;
        unsigned v[kScanItems];
        unsigned tsum = 0;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            v[j] = i0 + j < len ? counts[i0 + j] : 0u;
            tsum += v[j];
        }
        unsigned x = tsum;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) warp_tot[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned w = lane < (int)(blockDim.x >> 5) ? warp_tot[lane] : 0u;
            for (int o = 1; o < 32; o <<= 1) {
                const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            warp_tot[lane] = w;
        }
        __syncthreads();
        unsigned run = (warp > 0 ? warp_tot[warp - 1] : 0u) + carry + x - tsum;
#pragma unroll
        for (int j = 0; j < kScanItems; ++j) {
            if (i0 + j < len) counts[i0 + j] = run;
            run += v[j];
        }
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = run;
        __syncthreads();
    }
}

__global__ void sort_downsweep_kernel(const unsigned* __restrict__ keys_in, const unsigned* __restrict__ vals_in,
                                      unsigned* __restrict__ keys_out, unsigned* __restrict__ vals_out, int64_t n,
                                      int shift, const unsigned* __restrict__ offsets, int nblocks) {
    __shared__ unsigned wcount[kWarps][256];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int d = lane; d < 256; d += 32) wcount[warp][d] = 0;
    __syncwarp();
    // warp w owns elements [w*256, (w+1)*256) of the block tile, 32 at a time
    const int64_t base = static_cast<int64_t>(blockIdx.x) * kSortTile + warp * (kSortTile / kWarps);
    unsigned key[kSortItems], val[kSortItems], rank[kSortItems];
    const unsigned lt = (1u << lane) - 1u;
    for (int it = 0; it < kSortItems; ++it) {
        const int64_t i = base + it * 32 + lane;
        const bool valid = i < n;
        key[it] = valid ? keys_in[i] : 0u;
        val[it] = valid ? vals_in[i] : 0u;
        const unsigned dg = valid ? ((key[it] >> shift) & 0xFF) : 256u;
        const unsigned peers = __match_any_sync(0xffffffffu, dg);
        const unsigned r = __popc(peers & lt);
        unsigned prior = 0;
        if (valid) prior = wcount[warp][dg];
        rank[it] = prior + r;
        __syncwarp();
        if (valid && r == 0) wcount[warp][dg] = prior + __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    // per digit: exclusive prefix over warps
    {
        const int dg = threadIdx.x;  // 256 threads = 256 digits
        unsigned run = 0;
        for (int w = 0; w < kWarps; ++w) {
            const unsigned t = wcount[w][dg];
            wcount[w][dg] = run;
            run += t;
        }
    }
    __syncthreads();
    for (int it = 0; it < kSortItems; ++it) {
        const int64_t i = base + it * 32 + lane;
        if (i < n) {
            const unsigned dg = (key[it] >> shift) & 0xFF;
            const unsigned pos = offsets[static_cast<int64_t>(dg) * nblocks + blockIdx.x] + wcount[warp][dg] + rank[it];
            keys_out[pos] = key[it];
            vals_out[pos] = val[it];
        }
    }
}

// Column tiles from the sorted order (see layout above).
template <int DP>
__global__ void build_tiles_kernel(const float* __restrict__ xc, const float* __restrict__ norms, int64_t n, int d,
                                   const unsigned* __restrict__ perm, int64_t padded, float* __restrict__ tiles) {
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < padded;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t t = p / kCT;
        const int c = static_cast<int>(p % kCT);
        float* tile = tiles + t * tile_floats(DP);
        const bool valid = p < n;
        const unsigned orig = valid ? perm[p] : kNoIndex;
        const int pair = c >> 1, side = c & 1;
#pragma unroll
        for (int f = 0; f < DP; ++f) {
            const float v = (valid && f < d) ? xc[static_cast<int64_t>(orig) * d + f] : 0.0f;
            tile[pair * pair_stride(DP) + 2 * f + side] = v;
        }
        if (side == 0)
            for (int f = 2 * DP; f < pair_stride(DP); ++f) tile[pair * pair_stride(DP) + f] = 0.0f;
        tile[tile_norms_off(DP) + c] = valid ? norms[orig] : __int_as_float(0x7fc00000);
        reinterpret_cast<unsigned*>(tile)[tile_index_off(DP) + c] = orig;
    }
}

// ---------------------------------------------------------------- seed

// Exact distances (the oracle's formula: t = a - b, s = fma(t, t, s) over the
// dimensions in order) from row a (each coordinate duplicated into both
// halves) to the two columns of pair p of a tile, with packed f32x2
// instructions: per element the same IEEE operations as the scalar chain.
template <int DP>
__device__ __forceinline__ void pair_dist2(const float* tile, int p, const uint64_t (&a2)[DP], float& d0, float& d1) {
    uint64_t s = 0;  // (+0, +0)
#pragma unroll
    for (int f = 0; f < DP; ++f) {
        const uint64_t t = sub2(a2[f], *reinterpret_cast<const uint64_t*>(tile + p * pair_stride(DP) + 2 * f));
        s = fma2(t, t, s);
    }
    d0 = lo_f(s);
    d1 = hi_f(s);
}

// Per row of tile T: the exact k best keys over the seed window (sorted,
// kKeyMax padded) and its k-th key, the starting point of the row's shared
// k-th key (kth_shared) that the sweep CTAs tighten with atomicMin. The
// window is the first qs spiral positions: tile T itself and its Morton
// neighbours T+1, T-1, T+2 and T-2, whose points start the k-th distances much closer
// to their final values than tile T alone (fewer candidates reach the
// sweep's lists); the sweep covers the spiral from position qs on.
// Pruning margin: the float32 direct-difference distance D of two points at
// real squared distance T >= LB satisfies D >= T (1 - (d + 2) 2^-24) >
// LB (1 - 2^-20) for d <= 8, so a tile whose rounded-down box gap times
// (1 - 2^-20) exceeds every row's k-th distance holds no candidate.
constexpr float kPruneShrink = 0.99999904632568359375f;  // 1 - 2^-20

// One warp per tile: the bounding box of its valid points (the sweep's
// pruning test reads it with the tile).
template <int DP>
__global__ void tile_box_kernel(float* __restrict__ tiles, int nt, float* __restrict__ boxes) {
    const int lane = threadIdx.x & 31;
    const int t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (t >= nt) return;
    float* tile = tiles + static_cast<int64_t>(t) * tile_floats(DP);
    const unsigned* idx = reinterpret_cast<const unsigned*>(tile + tile_index_off(DP));
#pragma unroll
    for (int f = 0; f < DP; ++f) {
        float lo = __int_as_float(0x7f800000), hi = __int_as_float(0xff800000);
        for (int c = lane; c < kCT; c += 32) {
            if (idx[c] != kNoIndex) {
                const float v = tile_coord<DP>(tile, c, f);
                lo = fminf(lo, v);
                hi = fmaxf(hi, v);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            tile[tile_box_off(DP) + f] = lo;
            tile[tile_box_off(DP) + DP + f] = hi;
            boxes[static_cast<int64_t>(t) * 2 * DP + f] = lo;
            boxes[static_cast<int64_t>(t) * 2 * DP + DP + f] = hi;
        }
    }
}

// Squared distance between two boxes, rounded down (a lower bound of the
// real squared distance of any two points in them): lane f < DP takes
// dimension f, the sum runs with round-down additions. Warp-uniform result.
template <int DP>
__device__ __forceinline__ float box_gap2_rd(const float* __restrict__ a_lo, const float* __restrict__ a_hi,
                                             const float* __restrict__ b_lo, const float* __restrict__ b_hi) {
    const int lane = threadIdx.x & 31;
    float g = 0.0f;
    if (lane < DP) {
        const float g1 = __fsub_rd(b_lo[lane], a_hi[lane]);
        const float g2 = __fsub_rd(a_lo[lane], b_hi[lane]);
        const float gap = fmaxf(0.0f, fmaxf(g1, g2));
        g = __fmul_rd(gap, gap);
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) g = __fadd_rd(g, __shfl_xor_sync(0xffffffffu, g, o));
    return __shfl_sync(0xffffffffu, g, 0);
}

// Keys for the launch order of the sweep: 0xFFFF - list length (ascending
// sort = longest lists first), values the row tiles.
__global__ void order_key_kernel(const int* __restrict__ pcount, int t0, int mt, unsigned* __restrict__ keys,
                                 unsigned* __restrict__ vals) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= mt) return;
    keys[t] = 0xFFFFu - static_cast<unsigned>(pcount[t0 + t]);
    vals[t] = static_cast<unsigned>(t0 + t);
}

// Per row tile T (one block): the column tiles that can hold a candidate for
// any of its rows under the seed's k-th distances, in the sweep's visiting
// order, each with its rounded-down box gap (the sweep re-tests the gap
// against its tighter current k-th distances without touching the boxes).
template <int DP>
__global__ void __launch_bounds__(256) prune_list_kernel(const float* __restrict__ boxes, int nt, int t0, int qs,
                                                         const unsigned long long* __restrict__ kth_seed,
                                                         uint2* __restrict__ plist, int* __restrict__ pcount,
                                                         const float* __restrict__ tiles,
                                                         const unsigned char* __restrict__ iso_flag) {
    __shared__ float tbox[2][DP];
    __shared__ float wbox[4][2][DP];
    __shared__ float kmax_s;
    __shared__ int wtot[8];
    __shared__ int base_s;
    const int T = t0 + static_cast<int>(blockIdx.x);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (!iso_flag) {
        if (threadIdx.x < 2 * DP)
            tbox[threadIdx.x / DP][threadIdx.x % DP] = boxes[static_cast<int64_t>(T) * 2 * DP + threadIdx.x];
    } else if (warp < 4) {
        // the box of the rows that stay in the sweep (isolated rows take
        // their own pass; a tile with none gets an empty box)
        const float* own = tiles + static_cast<int64_t>(T) * tile_floats(DP);
        const int r = threadIdx.x;
        const bool keep = reinterpret_cast<const unsigned*>(own)[tile_index_off(DP) + r] != kNoIndex &&
                          !iso_flag[static_cast<int64_t>(T) * kRT + r];
#pragma unroll
        for (int f = 0; f < DP; ++f) {
            float lo = keep ? tile_coord<DP>(own, r, f) : __int_as_float(0x7f800000);
            float hi = keep ? tile_coord<DP>(own, r, f) : __int_as_float(0xff800000);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            }
            if (lane == 0) {
                wbox[warp][0][f] = lo;
                wbox[warp][1][f] = hi;
            }
        }
    }
    if (warp == 0) {
        const unsigned* own_idx =
            iso_flag ? reinterpret_cast<const unsigned*>(tiles + static_cast<int64_t>(T) * tile_floats(DP)) +
                           tile_index_off(DP)
                     : nullptr;
        float v = __int_as_float(0xff800000);
        for (int r = lane; r < kRT; r += 32) {
            const int64_t pos = static_cast<int64_t>(T) * kRT + r;
            if (iso_flag && (iso_flag[pos] || own_idx[r] == kNoIndex)) continue;  // not in the sweep
            const unsigned long long kk = kth_seed[pos];
            v = fmaxf(v, kk == kKeyMax ? __int_as_float(0x7f800000) : __uint_as_float(key_bits(kk)));
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        if (lane == 0) {
            kmax_s = v;
            base_s = 0;
        }
    }
    __syncthreads();
    if (iso_flag && threadIdx.x < DP) {
        const int f = threadIdx.x;
        tbox[0][f] = fminf(fminf(wbox[0][0][f], wbox[1][0][f]), fminf(wbox[2][0][f], wbox[3][0][f]));
        tbox[1][f] = fmaxf(fmaxf(wbox[0][1][f], wbox[1][1][f]), fmaxf(wbox[2][1][f], wbox[3][1][f]));
    }
    __syncthreads();
    const float kmax = kmax_s;
    uint2* out = plist + static_cast<int64_t>(T) * nt;
    for (int q0 = qs; q0 < nt; q0 += 256) {
        const int q = q0 + static_cast<int>(threadIdx.x);
        bool pass = false;
        unsigned t = 0;
        float g2 = 0.0f;
        if (q < nt) {
            t = static_cast<unsigned>(spiral_tile(T, q, nt));
            const float* b = boxes + static_cast<int64_t>(t) * 2 * DP;
#pragma unroll
            for (int f = 0; f < DP; ++f) {
                const float gap = fmaxf(0.0f, fmaxf(__fsub_rd(b[f], tbox[1][f]), __fsub_rd(tbox[0][f], b[DP + f])));
                g2 = __fadd_rd(g2, __fmul_rd(gap, gap));
            }
            pass = !(__fmul_rd(g2, kPruneShrink) > kmax);
        }
        const unsigned m = __ballot_sync(0xffffffffu, pass);
        if (lane == 0) wtot[warp] = __popc(m);
        __syncthreads();
        int before = base_s;
        for (int w = 0; w < warp; ++w) before += wtot[w];
        if (pass) out[before + __popc(m & ((1u << lane) - 1u))] = make_uint2(t, __float_as_uint(g2));
        __syncthreads();
        if (threadIdx.x == 0) {
            int tot = 0;
            for (int w = 0; w < 8; ++w) tot += wtot[w];
            base_s += tot;
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) pcount[T] = base_s;
}

template <int DP>
__global__ void __launch_bounds__(kThreads) seed_kernel(const float* __restrict__ tiles, int nt, int t0, int64_t n,
                                                        int k, int qs, uint64_t* __restrict__ seed_keys,
                                                        unsigned long long* __restrict__ kth_shared) {
    __shared__ __align__(16) float tile[kSeedWindow][tile_floats(DP)];
    __shared__ uint64_t wl[kWarps][96];  // per warp: the row's sorted k best (k <= 64), then up to 32 new keys
    const int T = t0 + static_cast<int>(blockIdx.x);
    for (int q = 0; q < qs; ++q) {
        const float* src = tiles + static_cast<int64_t>(spiral_tile(T, q, nt)) * tile_floats(DP);
        for (int i = threadIdx.x; i < tile_floats(DP); i += kThreads) tile[q][i] = src[i];
    }
    __syncthreads();
    const unsigned* idx = reinterpret_cast<const unsigned*>(tile[0] + tile_index_off(DP));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint64_t* lst = wl[warp];
    const auto exact = [](uint64_t key) { return key; };
    for (int r = warp; r < kRT; r += kWarps) {
        const int64_t pos = static_cast<int64_t>(T) * kRT + r;
        const bool row_valid = idx[r] != kNoIndex;
        uint64_t ra2[DP];  // the row's coordinates, duplicated for the packed chains
#pragma unroll
        for (int f = 0; f < DP; ++f) ra2[f] = dup2(tile_coord<DP>(tile[0], r, f));
        // own tile: its 128 keys (the k best of them sorted below); lane l
        // takes the columns of pairs l and l + 32
        uint64_t v[4];
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int p = h * 32 + lane;
            float d0, d1;
            pair_dist2<DP>(tile[0], p, ra2, d0, d1);
            const int c0 = 2 * p, c1 = 2 * p + 1;
            v[2 * h] = (row_valid && c0 != r && idx[c0] != kNoIndex) ? make_key(__float_as_uint(d0), idx[c0]) : kKeyMax;
            v[2 * h + 1] =
                (row_valid && c1 != r && idx[c1] != kNoIndex) ? make_key(__float_as_uint(d1), idx[c1]) : kKeyMax;
        }
        uint64_t kk = kKeyMax;
        uint64_t best = kKeyMax;  // k <= 32: the 32 best so far, sorted across the warp
        if (k <= 32) {
            // the first 32 keys sorted, the other three registers merged in
            // (those with a key below the current k-th key)
            uint64_t w[1] = {v[0]};
            warp_bitonic_sort<1>(w);
            best = w[0];
            kk = __shfl_sync(0xffffffffu, best, k - 1);
#pragma unroll
            for (int j = 1; j < 4; ++j) {
                if (!__any_sync(0xffffffffu, v[j] < kk)) continue;
                uint64_t x[1] = {v[j] < kk ? v[j] : kKeyMax};
                warp_bitonic_sort<1>(x);
                best = warp_merge_lowest32(best, x[0]);
                kk = __shfl_sync(0xffffffffu, best, k - 1);
            }
        } else {
            warp_bitonic_sort<4>(v);
            const int owner = (k - 1) & 31, oreg = (k - 1) >> 5;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const uint64_t t = __shfl_sync(0xffffffffu, v[j], owner);
                if (j == oreg) kk = t;
            }
        }
        if (row_valid && qs > 1 && k <= 32) {
            // neighbour tiles, k <= 32: the 32 best so far stay in one
            // register across the warp (sorted); keys below the current k-th
            // key gather in shared memory, 32 at most, and join by a bitonic
            // merge in registers
            int cnt = 0;
            const auto merge_pending = [&]() {
                uint64_t w[1] = {lane < cnt ? lst[lane] : kKeyMax};
                warp_bitonic_sort<1>(w);
                best = warp_merge_lowest32(best, w[0]);
                kk = __shfl_sync(0xffffffffu, best, k - 1);
                cnt = 0;
            };
            for (int q = 1; q < qs; ++q) {
                const unsigned* idq = reinterpret_cast<const unsigned*>(tile[q] + tile_index_off(DP));
                float dd[4];  // columns 2p and 2p + 1 of pairs p = l and l + 32
                pair_dist2<DP>(tile[q], lane, ra2, dd[0], dd[1]);
                pair_dist2<DP>(tile[q], lane + 32, ra2, dd[2], dd[3]);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = 2 * ((j >> 1) * 32 + lane) + (j & 1);
                    const uint64_t key = idq[c] != kNoIndex ? make_key(__float_as_uint(dd[j]), idq[c]) : kKeyMax;
                    unsigned m = __ballot_sync(0xffffffffu, key < kk);
                    if (m && cnt + __popc(m) > 32) {
                        __syncwarp();
                        merge_pending();
                        __syncwarp();
                        m = __ballot_sync(0xffffffffu, key < kk);
                    }
                    if (m) {
                        if (key < kk) lst[cnt + __popc(m & ((1u << lane) - 1u))] = key;
                        cnt += __popc(m);
                    }
                }
            }
            __syncwarp();
            if (cnt > 0) merge_pending();
            if (lane < k) seed_keys[pos * k + lane] = best;
            __syncwarp();
        } else if (row_valid && qs > 1) {
            // neighbour tiles: append the keys below the current k-th key and
            // merge them into the sorted k best (at most 32 at a time)
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int e = j * 32 + lane;
                if (e < k) lst[e] = v[j];
            }
            int cnt = k;
            for (int q = 1; q < qs; ++q) {
                const unsigned* idq = reinterpret_cast<const unsigned*>(tile[q] + tile_index_off(DP));
                float dd[4];  // columns 2p and 2p + 1 of pairs p = l and l + 32
                pair_dist2<DP>(tile[q], lane, ra2, dd[0], dd[1]);
                pair_dist2<DP>(tile[q], lane + 32, ra2, dd[2], dd[3]);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int c = 2 * ((j >> 1) * 32 + lane) + (j & 1);
                    const uint64_t key = idq[c] != kNoIndex ? make_key(__float_as_uint(dd[j]), idq[c]) : kKeyMax;
                    unsigned m = __ballot_sync(0xffffffffu, key < kk);
                    if (m && cnt + __popc(m) > k + 32) {
                        __syncwarp();
                        cnt = merge_sorted_prefix<1>(lst, k, cnt, k, k - 1, exact, &kk);
                        m = __ballot_sync(0xffffffffu, key < kk);
                    }
                    if (m) {
                        __syncwarp();
                        if (key < kk) lst[cnt + __popc(m & ((1u << lane) - 1u))] = key;
                        cnt += __popc(m);
                    }
                }
            }
            __syncwarp();
            if (cnt > k) cnt = merge_sorted_prefix<1>(lst, k, cnt, k, k - 1, exact, &kk);
            for (int e = lane; e < k; e += 32) seed_keys[pos * k + e] = lst[e];
            __syncwarp();
        } else if (k <= 32) {
            if (lane < k) seed_keys[pos * k + lane] = best;
        } else {
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const int e = j * 32 + lane;
                if (e < k) seed_keys[pos * k + e] = v[j];
            }
        }
        if (lane == 0) kth_shared[pos] = row_valid ? kk : kKeyMax;
    }
}

// ---------------------------------------------------------------- isolated rows
//
// A row whose seed k-th distance is among the largest (an isolated point:
// its neighbours are far away, so its warp of the sweep can prune almost no
// column tile) holds its warp busy on nearly every tile while the CTA's
// other warps skip most of them, and the CTA lasts as long as its busiest
// warp. About 1.2% of the rows, those with the largest seed k-th keys, leave
// the sweep (it treats them like padding rows) and take a pass of their
// own (iso_rows_kernel). Their result is the row's split-0 list, so the
// merge reads it like a sweep result. Which rows move is a performance
// choice only: every row's k best are exact either way.
constexpr int kIsoBins = 4096;        // histogram of seed k-th distances: their float bits >> 20
constexpr int kIsoBinShift = 20;
constexpr int kIsoPerMille = 12;      // about 1.2% of the rows leave
constexpr int kIsoMaxTiles = 8192;    // the pass keeps 4 gaps of 2 bytes per column tile in shared memory

// Histogram of the seed k-th distances of the valid positions [pos0, pos1)
// by the upper 12 bits of their float bits (sign, exponent, 3 mantissa
// bits: bins one eighth of an octave wide, in increasing order; a row with
// fewer than k neighbours in its seed window, k-th key kKeyMax, falls in
// the last bin); per-block counts in shared memory, then one atomic per
// non-empty bin. hist is zeroed by the caller.
__global__ void __launch_bounds__(256) iso_hist_kernel(const unsigned long long* __restrict__ kth_shared,
                                                       int64_t pos0, int64_t pos1, unsigned* __restrict__ hist) {
    __shared__ unsigned h[kIsoBins];
    for (int i = threadIdx.x; i < kIsoBins; i += blockDim.x) h[i] = 0;
    __syncthreads();
    for (int64_t pos = pos0 + static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; pos < pos1;
         pos += static_cast<int64_t>(gridDim.x) * blockDim.x)
        atomicAdd(&h[key_bits(kth_shared[pos]) >> kIsoBinShift], 1u);
    __syncthreads();
    for (int i = threadIdx.x; i < kIsoBins; i += blockDim.x)
        if (h[i]) atomicAdd(&hist[i], h[i]);
}

// One block: the lowest bin b whose rows and those of every higher bin
// number at most kIsoPerMille per mille of the valid rows (the highest bins first; at
// least one row): rows whose seed k-th key lies in bins >= b leave, so the
// threshold key is the last key below bin b. Also zeroes the row counter.
__global__ void __launch_bounds__(1024) iso_threshold_kernel(const unsigned* __restrict__ hist, int64_t rows,
                                                             unsigned long long* __restrict__ thr,
                                                             int* __restrict__ iso_count) {
    constexpr int kPer = kIsoBins / 1024;
    __shared__ unsigned part[1024];
    const int t = threadIdx.x;
    // this thread's bins are kPer consecutive ones from the top: bins
    // [kIsoBins - kPer (t + 1), kIsoBins - kPer t)
    unsigned own = 0;
#pragma unroll
    for (int j = 0; j < kPer; ++j) own += hist[kIsoBins - kPer * (t + 1) + j];
    part[t] = own;
    __syncthreads();
    // inclusive scan from the top (Hillis-Steele over the 1024 partial sums)
    for (int o = 1; o < 1024; o <<= 1) {
        const unsigned v = t >= o ? part[t - o] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    const int64_t target = rows * kIsoPerMille / 1000 > 0 ? rows * kIsoPerMille / 1000 : 1;
    const unsigned above = t > 0 ? part[t - 1] : 0u;  // rows in the bins above this thread's
    // the thread whose bins take the running count past the target picks
    // the lowest of its bins that keeps it within the target
    if (above <= target && part[t] > target) {
        unsigned run = above;
        int b = kIsoBins - kPer * t;  // one past this thread's highest bin
        for (int j = kPer - 1; j >= 0; --j) {
            const int bin = kIsoBins - kPer * (t + 1) + j;
            if (run + hist[bin] > target) break;
            run += hist[bin];
            b = bin;
        }
        *thr = b >= kIsoBins ? ~0ull  // the top bin alone is past the target: no row leaves
                             : (static_cast<unsigned long long>(static_cast<unsigned>(b) << kIsoBinShift) << 32) - 1ull;
    }
    if (t == 0) {
        if (part[1023] <= target) *thr = 0ull;  // every row (only for a handful of rows)
        *iso_count = 0;
    }
}

// Positions [pos0, pend) of the row tiles: flag[pos] = 1 for the valid rows
// (pos < n) whose seed k-th key exceeds the threshold, up to cap of them,
// and their positions listed (in no particular order; *iso_count may pass
// cap, the list holds min(*iso_count, cap)).
__global__ void iso_mark_kernel(const unsigned long long* __restrict__ kth_shared, int64_t pos0, int64_t pend,
                                int64_t n, const unsigned long long* __restrict__ thr, int cap,
                                unsigned char* __restrict__ flag, int* __restrict__ iso_list,
                                int* __restrict__ iso_count) {
    const unsigned long long t = *thr;
    const int lane = threadIdx.x & 31;
    for (int64_t b = pos0 + static_cast<int64_t>(blockIdx.x) * blockDim.x; b < pend;
         b += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t pos = b + threadIdx.x;
        bool iso = pos < pend && pos < n && kth_shared[pos] > t;
        const unsigned m = __ballot_sync(0xffffffffu, iso);
        if (m) {
            const int leader = __ffs(m) - 1;
            int base = 0;
            if (lane == leader) base = atomicAdd(iso_count, __popc(m));
            base = __shfl_sync(0xffffffffu, base, leader);
            const int slot = base + __popc(m & ((1u << lane) - 1u));
            iso = iso && slot < cap;
            if (iso) iso_list[slot] = static_cast<int>(pos);
        }
        if (pos < pend) flag[pos] = iso ? 1 : 0;
    }
}

// The k best keys below a bound, kept by one warp: for k <= 32 the 32 best
// so far sorted across the warp (one per lane) with up to 32 pending keys in
// shared memory; for k > 32 a sorted prefix of at most k keys plus up to 32
// new ones in shared memory (buf holds 96 keys). bound only decreases: the
// smaller of the caller's bound and the k-th key held.
// Out of line (one copy of the sorting networks for every call site): merges
// the pending keys of a WarpBest (see below) and tightens its bound.
__device__ __noinline__ void warp_best_flush(uint64_t* buf, int k, uint64_t& bound, uint64_t& best, int& cnt,
                                             int& sorted) {
    const int lane = threadIdx.x & 31;
    if (k <= 32) {
        uint64_t w[1] = {lane < cnt ? buf[lane] : kKeyMax};
        warp_bitonic_sort<1>(w);
        best = warp_merge_lowest32(best, w[0]);
        const uint64_t kth = __shfl_sync(0xffffffffu, best, k - 1);
        bound = kth < bound ? kth : bound;
        cnt = 0;
    } else {
        uint64_t sel;
        cnt = merge_sorted_prefix<1>(buf, sorted, cnt, k, k - 1, [](uint64_t key) { return key; }, &sel);
        sorted = cnt;
        bound = sel < bound ? sel : bound;
    }
    __syncwarp();
}

struct WarpBest {
    uint64_t* buf;
    int k;
    uint64_t bound;
    uint64_t best = kKeyMax;
    int cnt = 0;     // k <= 32: pending keys; k > 32: buffer length
    int sorted = 0;  // k > 32: buf[0..sorted) is sorted

    __device__ __forceinline__ void flush() { warp_best_flush(buf, k, bound, best, cnt, sorted); }
    // every lane offers one key (kKeyMax: none)
    __device__ __forceinline__ void offer(uint64_t key) {
        const int lane = threadIdx.x & 31;
        unsigned m = __ballot_sync(0xffffffffu, key < bound);
        if (m && cnt + __popc(m) > (k <= 32 ? 32 : sorted + 32)) {
            __syncwarp();
            flush();
            m = __ballot_sync(0xffffffffu, key < bound);
        }
        if (m) {
            if (key < bound) buf[cnt + __popc(m & ((1u << lane) - 1u))] = key;
            cnt += __popc(m);
            __syncwarp();
        }
    }
    __device__ __forceinline__ void finish() {
        if (cnt > (k <= 32 ? 0 : sorted)) flush();
    }
    // after finish(): key e of the k best (sorted ascending, kKeyMax padded);
    // for k <= 32 only lane e's own element (e == lane) is available
    __device__ __forceinline__ uint64_t get(int e) const {
        if (k <= 32) return best;
        return e < sorted ? buf[e] : kKeyMax;
    }
};

// Quarter tiles: the pass prunes 32-column quarters of a tile (tighter
// boxes than whole tiles around isolated points) and reads a dimension-major
// copy of the column coordinates, so one quarter is DP coalesced 128-byte
// loads: cols[(t * DP + f) * kCT + c] = coordinate f of column c of tile t.
constexpr int kQuarter = 32;
constexpr int kQuarters = kCT / kQuarter;

template <int DP>
__global__ void iso_cols_kernel(const float* __restrict__ tiles, int nt, float* __restrict__ cols) {
    const int64_t total = static_cast<int64_t>(nt) * DP * kCT;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < total;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t t = i / (DP * kCT);
        const int f = static_cast<int>(i / kCT % DP), c = static_cast<int>(i % kCT);
        cols[i] = tile_coord<DP>(tiles + t * tile_floats(DP), c, f);
    }
}

// One warp per quarter: the bounding box of its valid columns as a 32-byte
// record of 16 bf16 values, qbox[16 q + f] = lower bound of dimension f
// rounded down, qbox[16 q + 8 + f] = upper bound rounded up (a box that
// contains the float32 one; +inf / -inf when the quarter has no valid
// column; unused slots 0), for quarter q = 4 t + j.
template <int DP>
__global__ void iso_qbox_kernel(const float* __restrict__ tiles, const float* __restrict__ cols, int nt,
                                __nv_bfloat16* __restrict__ qbox) {
    const int lane = threadIdx.x & 31;
    const int64_t nq = static_cast<int64_t>(nt) * kQuarters;
    for (int64_t q = (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) / 32; q < nq;
         q += static_cast<int64_t>(gridDim.x) * blockDim.x / 32) {
        const int64_t t = q / kQuarters;
        const int c = static_cast<int>(q % kQuarters) * kQuarter + lane;
        const bool valid =
            reinterpret_cast<const unsigned*>(tiles + t * tile_floats(DP))[tile_index_off(DP) + c] != kNoIndex;
        float mine = 0.0f;  // lane f: lower bound of dimension f; lane 8 + f: upper bound
#pragma unroll
        for (int f = 0; f < DP; ++f) {
            const float v = cols[(t * DP + f) * kCT + c];
            float lo = valid ? v : __int_as_float(0x7f800000), hi = valid ? v : __int_as_float(0xff800000);
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) {
                lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
                hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
            }
            if (lane == f) mine = lo;
            if (lane == 8 + f) mine = hi;
        }
        if (lane < 16)
            qbox[16 * q + lane] = lane < 8 ? __float2bfloat16_rd(mine) : __float2bfloat16_ru(mine);
    }
}

// Gaps are kept as the upper 16 bits of their float32 bit pattern
// (non-negative floats truncated: rounded down, so pruning stays
// conservative); kGapSkip marks a quarter the pass never visits.
constexpr uint16_t kGapSkip = 0xFFFFu;
__device__ __forceinline__ uint16_t gap_bits_down(float g) { return static_cast<uint16_t>(__float_as_uint(g) >> 16); }
// the smallest 16-bit pattern not below distance b (+inf: 0x7F80)
__device__ __forceinline__ unsigned bound_bits_up(float b) { return (__float_as_uint(b) + 0xFFFFu) >> 16; }

// One warp: up to kIsoBatch quarters q[0..m) against point a (the seed's
// exact arithmetic: dimensions in order), every key offered. Lane l takes
// column l of each quarter; all loads are issued first.
constexpr int kIsoBatch = 4;
template <int DP>
__device__ __forceinline__ void iso_eval_quarters(const float* __restrict__ tiles, const float* __restrict__ cols,
                                                  const int (&q)[kIsoBatch], int m, const float (&a)[DP],
                                                  WarpBest& wb) {
    const int lane = threadIdx.x & 31;
    float x[kIsoBatch][DP];
    unsigned ix[kIsoBatch];
#pragma unroll
    for (int i = 0; i < kIsoBatch; ++i) {
        const int qi = q[i < m ? i : 0];
        const int64_t t = qi / kQuarters;
        const int c = (qi % kQuarters) * kQuarter + lane;
#pragma unroll
        for (int f = 0; f < DP; ++f) x[i][f] = cols[(t * DP + f) * kCT + c];
        ix[i] = reinterpret_cast<const unsigned*>(tiles + t * tile_floats(DP))[tile_index_off(DP) + c];
    }
#pragma unroll
    for (int i = 0; i < kIsoBatch; ++i) {
        if (i >= m) break;
        float d2 = 0.0f;
#pragma unroll
        for (int f = 0; f < DP; ++f) {
            const float t = __fsub_rn(a[f], x[i][f]);
            d2 = __fmaf_rn(t, t, d2);
        }
        wb.offer(ix[i] != kNoIndex ? make_key(__float_as_uint(d2), ix[i]) : kKeyMax);
    }
}

// One CTA (kIsoWarps warps) per listed row: its k best keys (sorted,
// kKeyMax padded) over the column tiles outside the seed window of its row
// tile, below its seed k-th key, written to out[pos * k ..].
//  1. The rounded-down gap between the point and every quarter's box
//     (coalesced, into shared memory; the window's quarters are skipped).
//  2. Warp w owns quarter w of every tile (the quarters near the point are
//     spread over all warps) and visits its quarters in three rounds of
//     growing gap: gaps up to 1/16 of the row's current bound, then 1/4,
//     then the whole bound, so that the bound tightens on the nearest
//     quarters before the far ones are tested; quarters within the bound
//     are evaluated kIsoBatch at a time.
//  3. The warps share the bound (the smallest of the seed's k-th key and
//     their own k-th keys) in shared memory and merge their lists at the
//     end.
constexpr int kIsoWarps = 4;
template <int DP>
__global__ void __launch_bounds__(32 * kIsoWarps, 6) iso_rows_kernel(const float* __restrict__ tiles,
                                                                    const float* __restrict__ cols,
                                                                    const __nv_bfloat16* __restrict__ qbox, int nt, int qs,
                                                                    int k, int cap, const int* __restrict__ iso_list,
                                                                    const int* __restrict__ iso_count,
                                                                    const unsigned long long* __restrict__ kth_shared,
                                                                    uint64_t* __restrict__ out) {
    extern __shared__ __align__(16) uint16_t qgap_s[];  // 4 per tile
    __shared__ uint64_t wl[kIsoWarps][96];              // per warp: WarpBest's buffer
    __shared__ uint64_t fin[kIsoWarps][kMaxK];         // per warp: its k best at the end
    __shared__ unsigned long long bound_s;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int count = min(*iso_count, cap);
    const int nb = (nt + 31) / 32;
    const int64_t nq = static_cast<int64_t>(nt) * kQuarters;
    // the seed window: spiral positions 0..qs-1, offsets -(qs-1)/2 .. qs/2
    const int wlo = (qs - 1) / 2, whi = qs / 2;
    for (int h = blockIdx.x; h < count; h += gridDim.x) {
        const int64_t pos = iso_list[h];
        const int T = static_cast<int>(pos / kRT), r = static_cast<int>(pos % kRT);
        const float* own = tiles + static_cast<int64_t>(T) * tile_floats(DP);
        float a[DP];
#pragma unroll
        for (int f = 0; f < DP; ++f) a[f] = tile_coord<DP>(own, r, f);
        if (threadIdx.x == 0) bound_s = kth_shared[pos];
#pragma unroll 4
        for (int q = threadIdx.x; q < nq; q += 32 * kIsoWarps) {
            const int t = q / kQuarters;
            int off = t - T;  // offset from the row tile, in (-nt/2, nt/2]
            if (off > nt / 2) off -= nt;
            if (off <= -((nt + 1) / 2)) off += nt;
            const uint4 lo4 = reinterpret_cast<const uint4*>(qbox)[2 * q];
            const uint4 hi4 = reinterpret_cast<const uint4*>(qbox)[2 * q + 1];
            const unsigned lw[4] = {lo4.x, lo4.y, lo4.z, lo4.w}, hw[4] = {hi4.x, hi4.y, hi4.z, hi4.w};
            float g2 = 0.0f;
#pragma unroll
            for (int f = 0; f < DP; ++f) {  // bf16 to float is exact: the bits shifted up
                const float lo = __uint_as_float((f & 1 ? lw[f >> 1] >> 16 : lw[f >> 1] & 0xFFFFu) << 16);
                const float hi = __uint_as_float((f & 1 ? hw[f >> 1] >> 16 : hw[f >> 1] & 0xFFFFu) << 16);
                const float gap = fmaxf(0.0f, fmaxf(__fsub_rd(lo, a[f]), __fsub_rd(a[f], hi)));
                g2 = __fadd_rd(g2, __fmul_rd(gap, gap));
            }
            qgap_s[q] = (off >= -wlo && off <= whi) ? kGapSkip : gap_bits_down(__fmul_rd(g2, kPruneShrink));
        }
        __syncthreads();
        WarpBest wb{wl[warp], k, bound_s};
        const auto shared_bound = [&]() {  // publish this warp's bound, take the CTA's
            uint64_t sb = 0;
            if (lane == 0) sb = atomicMin(&bound_s, static_cast<unsigned long long>(wb.bound));
            sb = __shfl_sync(0xffffffffu, sb, 0);
            if (sb < wb.bound) wb.bound = sb;
        };
        const auto bound_up = [&]() {
            return wb.bound == kKeyMax ? 0xFFFEu : bound_bits_up(__uint_as_float(key_bits(wb.bound)));
        };
        int batch[kIsoBatch];  // quarters waiting for evaluation (warp-uniform)
        int nbatch = 0;
        unsigned lo_bits = 0;  // this round takes tiles whose gap lies in [lo_bits, hi_bits]
        for (int round = 0; round < 3; ++round) {
            shared_bound();
            const float bd = wb.bound == kKeyMax ? __int_as_float(0x7f800000) : __uint_as_float(key_bits(wb.bound));
            const float frac = round == 0 ? 0.0625f : round == 1 ? 0.25f : 1.0f;
            unsigned hi_bits = bound_bits_up(bd * frac);
            if (round == 2 || hi_bits > 0xFFFEu) hi_bits = 0xFFFEu;  // the last round takes every quarter left
            if (hi_bits < lo_bits) continue;
            for (int b = 0; b < nb; ++b) {
                const int t = 32 * b + lane;
                const unsigned g = t < nt ? qgap_s[kQuarters * t + warp] : kGapSkip;
                unsigned todo = __ballot_sync(0xffffffffu, g >= lo_bits && g <= hi_bits && g <= bound_up());
                while (todo) {
                    const int src = __ffs(todo) - 1;
                    todo &= todo - 1;
                    if (__shfl_sync(0xffffffffu, g, src) > bound_up()) continue;  // a tighter bound prunes it
                    batch[nbatch++] = (32 * b + src) * kQuarters + warp;
                    if (nbatch == kIsoBatch) {
                        iso_eval_quarters<DP>(tiles, cols, batch, nbatch, a, wb);
                        nbatch = 0;
                        shared_bound();
                    }
                }
            }
            lo_bits = hi_bits + 1;
        }
        if (nbatch > 0) iso_eval_quarters<DP>(tiles, cols, batch, nbatch, a, wb);
        wb.finish();
        for (int e = lane; e < k; e += 32) fin[warp][e] = wb.get(e);
        __syncthreads();
        // warp 0 merges the other warps' lists into its own, under the seed's
        // k-th key (the shared bound may equal a key of those lists)
        if (warp == 0) {
            wb.bound = kth_shared[pos];
            for (int w = 1; w < kIsoWarps; ++w)
                for (int e0 = 0; e0 < k; e0 += 32) {
                    const int e = e0 + lane;
                    wb.offer(e < k ? fin[w][e] : kKeyMax);
                }
            wb.finish();
            uint64_t* dst = out + pos * k;
            for (int e = lane; e < k; e += 32) dst[e] = wb.get(e);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- sweep

template <int DP, int M>
struct SweepSmem {
    union {
        float tiles[kStages][tile_floats(DP)];
        // (-2a, -2a) per row and dimension, the packed FMA operands: every
        // warp copies its rows into registers before the barrier that
        // precedes the first tile copy, so they share the tiles' space
        uint64_t rowd[kRT][DP];
    };
    RowLists<M> L;
    uint64_t full_bar[kStages];
    float rowc[kRT][DP];
    int done[kStages];
    uint16_t queue[kWarps][kQueueCap];
    float wbox[kWarps][2][DP];  // bounding box of each warp's 16 rows
    float wkmax[kWarps];        // largest k-th distance among each warp's rows
    float cbox[2][DP];          // bounding box of the CTA's rows
    int stage_tile[kStages];    // column tile in each stage, -1: the split is done
    int last_fill[kStages];     // fill number of the stage's last tile copy (-1: none)
    int next_j;                 // the loader's scan position in the split's sequence
    unsigned evaluated;         // warp x column-tile blocks evaluated (not pruned)
};


// Exact rescoring of the warp's queued candidates (one per lane): exact
// distance, append to the row list if the key beats the row's k-th key;
// rows that are filling up are compacted after every chunk of 32 (so a list
// never overflows: M >= k + 32). Returns true if any row was compacted.
template <int DP, int M>
__device__ bool drain_queue(SweepSmem<DP, M>& sh, int qc, const float* __restrict__ tl, int k, float nmax) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned* tidx = reinterpret_cast<const unsigned*>(tl + tile_index_off(DP));
    bool compacted = false;
    for (int base = 0; base < qc; base += 32) {
        const int i = base + lane;
        if (i < qc) {
            const unsigned e = sh.queue[warp][i];
            const int r = static_cast<int>(e >> 8), c = static_cast<int>(e & 0xFF);
            float s = 0.0f;
#pragma unroll
            for (int f = 0; f < DP; ++f) {
                const float t = __fsub_rn(sh.rowc[r][f], tile_coord<DP>(tl, c, f));
                s = __fmaf_rn(t, t, s);
            }
            const uint64_t key = make_key(__float_as_uint(s), tidx[c]);
            if (key < sh.L.kth[r]) {
                const int slot = atomicAdd(&sh.L.cnt[r], 1);
                sh.L.list[r][slot] = key;
            }
        }
        __syncwarp();
        compacted |= compact_full_rows<M>(sh.L, k, nmax, DP);
    }
    return compacted;
}

// One CTA per (row tile T, split): the rows of T against the split's share
// of the other column tiles. Each warp owns 16 rows (their lists, k-th keys
// and thresholds), so list maintenance needs no block barrier; column tiles
// arrive by TMA and the last warp to finish a tile refills its stage.
template <int DP, int M>
__global__ void __launch_bounds__(kThreads, 2)
sweep_kernel(const float* __restrict__ tiles, int nt, int t0, int mt, int qs, int nsplit, int k,
             const unsigned* __restrict__ max_norm_bits,
             unsigned long long* __restrict__ kth_shared, uint64_t* __restrict__ partial, int* __restrict__ status,
             unsigned long long* __restrict__ evaluated_blocks, const uint2* __restrict__ plist,
             const int* __restrict__ pcount, const unsigned* __restrict__ order, const float* __restrict__ boxes,
             const unsigned char* __restrict__ iso_flag) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    SweepSmem<DP, M>& sh = *reinterpret_cast<SweepSmem<DP, M>*>(smem_raw);
    // row tiles with the longest candidate lists first (tail balance)
    // (split-major: a row tile's later splits start after its earlier ones
    // have shared their k-th keys, so they prune more)
    // (row tiles [t0, t0 + mt) of the nt: a shard of the rows)
    const int ti = static_cast<int>(blockIdx.x) % mt;
    const int T = order ? static_cast<int>(order[ti]) : t0 + ti;
    const int split = static_cast<int>(blockIdx.x) / mt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float nmax = __uint_as_float(*max_norm_bits);
    const float* own = tiles + static_cast<int64_t>(T) * tile_floats(DP);
    // this split's share of the row tile's candidate column tiles: entries
    // split + nsplit j of its list (visiting order, interleaved, so every
    // split meets the nearby tiles first)
    // (without lists, very large n: every tile past the seed window in
    // spiral order)
    const int lcount = plist ? pcount[T] : nt - qs;
    const int count = lcount > split ? (lcount - split + nsplit - 1) / nsplit : 0;
    const uint2* tlist = plist ? plist + static_cast<int64_t>(T) * nt : nullptr;
    constexpr unsigned kTileBytes = tile_bytes(DP);

    if (tid < kRT) {
        const int64_t pos = static_cast<int64_t>(T) * kRT + tid;
        const float nr = own[tile_norms_off(DP) + tid];
        const uint64_t kk = kth_shared[pos];
        sh.L.kth[tid] = kk;
        sh.L.row_norm[tid] = nr;
        // padding rows and isolated rows (their own pass) take no candidates
        sh.L.tau[tid] = (reinterpret_cast<const unsigned*>(own)[tile_index_off(DP) + tid] == kNoIndex ||
                         (iso_flag && iso_flag[pos]))
                          ? __int_as_float(0xff800000)
                          : tau_from(kk, nr, nmax, DP);
        sh.L.cnt[tid] = 0;
        sh.L.sorted[tid] = 0;
#pragma unroll
        for (int f = 0; f < DP; ++f) {
            sh.rowc[tid][f] = tile_coord<DP>(own, tid, f);
            sh.rowd[tid][f] = dup2(-2.0f * sh.rowc[tid][f]);
        }
    }
    if (tid < kStages) {
        sh.done[tid] = 0;
        sh.last_fill[tid] = -1;
    }
    if (tid == 0) {
        sh.evaluated = 0;
        sh.next_j = 0;
        for (int s = 0; s < kStages; ++s) mbar_init(&sh.full_bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // lane = (row group g, pair slot cp): rows warp*16 + g*4 + j, pairs s*8 + cp
    const int g = lane >> 3, cp = lane & 7;
    const int rbase = warp * kRowsPerWarp + g * kRowsPerLane;
    uint64_t a2[kRowsPerLane][DP];
    float tau_r[kRowsPerLane];
    uint64_t tau2[kRowsPerLane];  // dup(next float above tau): e <= tau  <=>  sign(e - tau') set
#pragma unroll
    for (int j = 0; j < kRowsPerLane; ++j) {
#pragma unroll
        for (int f = 0; f < DP; ++f) {
            // Loaded as 64-bit pairs from shared memory: the compiler cannot see
            // that both halves are equal, so each operand stays a register pair
            // for the whole sweep (rebuilding the pair costs a move per FMA).
            a2[j][f] = sh.rowd[rbase + j][f];
        }
        tau_r[j] = sh.L.tau[rbase + j];
        tau2[j] = dup2(tau_above(tau_r[j]));
    }
    // this warp's row box and the largest k-th distance among its rows
    // (invalid rows take no candidates and do not count)
    const unsigned* own_idx = reinterpret_cast<const unsigned*>(own) + tile_index_off(DP);
    const int wrow = warp * kRowsPerWarp + (lane & 15);
    const bool wvalid =
        own_idx[wrow] != kNoIndex && !(iso_flag && iso_flag[static_cast<int64_t>(T) * kRT + wrow]);
#pragma unroll
    for (int f = 0; f < DP; ++f) {
        float lo = wvalid ? sh.rowc[wrow][f] : __int_as_float(0x7f800000);
        float hi = wvalid ? sh.rowc[wrow][f] : __int_as_float(0xff800000);
#pragma unroll
        for (int o = 8; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            sh.wbox[warp][0][f] = lo;
            sh.wbox[warp][1][f] = hi;
        }
    }
    auto warp_kth = [&]() -> float {
        const uint64_t kk = sh.L.kth[wrow];
        float v = !wvalid ? __int_as_float(0xff800000)
                          : (kk == kKeyMax ? __int_as_float(0x7f800000) : __uint_as_float(key_bits(kk)));
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
        return v;
    };
    __syncwarp();
    float wk = warp_kth();
    if (lane == 0) sh.wkmax[warp] = wk;

    // The stage loader (one warp at a time): the next column tile of the
    // split that can hold a candidate for some row of this CTA, tested 32 at
    // a time against the CTA's row box and largest k-th distance (stale
    // values only prune less); a stage with no tile left gets a sentinel.
    auto fill = [&](int stage, int fill_no) {
        float kmax = lane < kWarps ? sh.wkmax[lane] : __int_as_float(0xff800000);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) kmax = fmaxf(kmax, __shfl_xor_sync(0xffffffffu, kmax, o));
        int found = -1;
        int base = sh.next_j;
        while (found < 0 && base < count) {
            const int j = base + lane;
            int t = -1;
            bool pass = false;
            if (j < count) {
                if (tlist) {
                    const uint2 e = __ldg(tlist + split + nsplit * j);
                    t = static_cast<int>(e.x);
                    pass = !(__fmul_rd(__uint_as_float(e.y), kPruneShrink) > kmax);
                } else {
                    // no list: the tile's own box (global array, the
                    // list builder's rounded-down gap) against the CTA box
                    t = spiral_tile(T, qs + split + nsplit * j, nt);
                    const float* b = boxes + static_cast<int64_t>(t) * 2 * DP;
                    float g2 = 0.0f;
#pragma unroll 1
                    for (int f = 0; f < DP; ++f) {  // rolled: the row registers are live here
                        const float gap =
                            fmaxf(0.0f, fmaxf(__fsub_rd(b[f], sh.cbox[1][f]), __fsub_rd(sh.cbox[0][f], b[DP + f])));
                        g2 = __fadd_rd(g2, __fmul_rd(gap, gap));
                    }
                    pass = !(__fmul_rd(g2, kPruneShrink) > kmax);
                }
            }
            const unsigned mk = __ballot_sync(0xffffffffu, pass);
            if (mk) {
                const int o = __ffs(mk) - 1;
                found = __shfl_sync(0xffffffffu, t, o);
                base += o + 1;
            } else {
                base += 32;
            }
        }
        if (lane == 0) {
            sh.next_j = base;
            if (found >= 0) {
                sh.stage_tile[stage] = found;
                sh.last_fill[stage] = fill_no;
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                mbar_expect_tx(&sh.full_bar[stage], kTileBytes);
                tma_load_1d(sh.tiles[stage], tiles + static_cast<int64_t>(found) * tile_floats(DP), kTileBytes,
                            &sh.full_bar[stage]);
            } else {
                sh.stage_tile[stage] = -1;
                mbar_arrive_plain(&sh.full_bar[stage]);
            }
        }
        __syncwarp();
    };
    __syncthreads();
    if (tid < DP) {
        float lo = __int_as_float(0x7f800000), hi = __int_as_float(0xff800000);
        for (int w = 0; w < kWarps; ++w) {
            lo = fminf(lo, sh.wbox[w][0][tid]);
            hi = fmaxf(hi, sh.wbox[w][1][tid]);
        }
        sh.cbox[0][tid] = lo;
        sh.cbox[1][tid] = hi;
    }
    __syncthreads();
    if (warp == 0)
        for (int st = 0; st < kStages; ++st) fill(st, st);

    bool ok = true;
    unsigned evaluated = 0;  // this warp's evaluated (not pruned) column tiles
    for (int m = 0; ok; ++m) {
        const int stage = m % kStages;
        if (!mbar_wait_warp(&sh.full_bar[stage], (m / kStages) & 1)) {
            ok = false;
            break;
        }
        if (sh.stage_tile[stage] < 0) break;  // the split is done
        const float* tl = sh.tiles[stage];
        const float* tn = tl + tile_norms_off(DP);
        int qc = 0;
        // prune: the whole tile is farther than every row's k-th distance
        const float* tb = tl + tile_box_off(DP);
        const bool skip = __fmul_rd(box_gap2_rd<DP>(sh.wbox[warp][0], sh.wbox[warp][1], tb, tb + DP), kPruneShrink) > wk;
        evaluated += skip ? 0u : 1u;
#pragma unroll 2
        for (int s = 0; s < (skip ? 0 : kPairs / 8); ++s) {
            const int p = s * 8 + cp;
            uint64_t B[DP];
#pragma unroll
            for (int f = 0; f < DP; f += 2) {
                const ulonglong2 v = *reinterpret_cast<const ulonglong2*>(tl + p * pair_stride(DP) + 2 * f);
                B[f] = v.x;
                B[f + 1] = v.y;
            }
            const uint64_t nb = *reinterpret_cast<const uint64_t*>(tn + 2 * p);
            uint64_t acc[kRowsPerLane];
#pragma unroll
            for (int j = 0; j < kRowsPerLane; ++j) acc[j] = nb;
#pragma unroll
            for (int f = 0; f < DP; ++f) {
#pragma unroll
                for (int j = 0; j < kRowsPerLane; ++j) acc[j] = fma2(a2[j][f], B[f], acc[j]);
            }
            // any of the 8 pairs below its row's threshold? One packed subtract per
            // row and an OR of the sign bits (e - tau' < 0 exactly when e < tau').
            unsigned signs = 0;
#pragma unroll
            for (int j = 0; j < kRowsPerLane; ++j) {
                const uint64_t dlt = sub2(acc[j], tau2[j]);
                signs |= static_cast<unsigned>(dlt) | static_cast<unsigned>(dlt >> 32);
            }
            if (__any_sync(0xffffffffu, static_cast<int>(signs) < 0)) {
                unsigned pass = 0;
#pragma unroll
                for (int j = 0; j < kRowsPerLane; ++j) {
                    pass |= (lo_f(acc[j]) <= tau_r[j] ? 1u : 0u) << (2 * j);
                    pass |= (hi_f(acc[j]) <= tau_r[j] ? 1u : 0u) << (2 * j + 1);
                }
                // queue (row, column) of every passing pair; warp-ordered slots
                const int cntp = __popc(pass);
                int off = cntp;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xffffffffu, off, o);
                    if (lane >= o) off += y;
                }
                const int tot = __shfl_sync(0xffffffffu, off, 31);
                off -= cntp;
                while (pass) {
                    const int b = __ffs(pass) - 1;
                    pass &= pass - 1;
                    const int r = rbase + (b >> 1);
                    const int c = 2 * p + (b & 1);
                    sh.queue[warp][qc + off++] = static_cast<uint16_t>((r << 8) | c);
                }
                qc += tot;
                __syncwarp();
                if (qc >= 32) {
                    if (drain_queue<DP, M>(sh, qc, tl, k, nmax)) {
#pragma unroll
                        for (int j = 0; j < kRowsPerLane; ++j) {
                            tau_r[j] = sh.L.tau[rbase + j];
                            tau2[j] = dup2(tau_above(tau_r[j]));
                        }
                        wk = warp_kth();
                        if (lane == 0) sh.wkmax[warp] = wk;
                    }
                    qc = 0;
                }
            }
        }
        if (qc > 0) {
            if (drain_queue<DP, M>(sh, qc, tl, k, nmax)) {
#pragma unroll
                for (int j = 0; j < kRowsPerLane; ++j) {
                    tau_r[j] = sh.L.tau[rbase + j];
                    tau2[j] = dup2(tau_above(tau_r[j]));
                }
                wk = warp_kth();
                if (lane == 0) sh.wkmax[warp] = wk;
            }
        }
        // done with this stage; the last warp out refills it
        __syncwarp();
        int prev = 0;
        if (lane == 0) {
            __threadfence_block();
            prev = atomicAdd(&sh.done[stage], 1);
        }
        prev = __shfl_sync(0xffffffffu, prev, 0);
        if (prev == kWarps - 1) {
            if (lane == 0) sh.done[stage] = 0;
            fill(stage, m + kStages);
        }
    }
    if (lane == 0) atomicAdd(&sh.evaluated, evaluated);
    const int failed = __syncthreads_or(ok ? 0 : 1);
    if (tid == 0 && evaluated_blocks) atomicAdd(evaluated_blocks, static_cast<unsigned long long>(sh.evaluated));
    if (failed) {
        if (tid == 0) atomicExch(status, 1);
        // wait (bounded) for this CTA's copies still in flight before exiting
        if (tid < kStages && sh.last_fill[tid] >= 0) mbar_wait(&sh.full_bar[tid], (sh.last_fill[tid] / kStages) & 1);
        __syncthreads();
        return;
    }
    // final: this split's sorted k best per row; share the k-th key (an
    // isolated row's split-0 list is written by its own pass)
    for (int i = 0; i < kRowsPerWarp; ++i) {
        const int r = warp * kRowsPerWarp + i;
        if (split == 0 && iso_flag && iso_flag[static_cast<int64_t>(T) * kRT + r]) continue;
        compact_row<M>(sh.L, r, k, nmax, DP);
        const int64_t pos = static_cast<int64_t>(T) * kRT + r;
        const int c = sh.L.cnt[r];
        uint64_t* out = partial + (static_cast<int64_t>(split) * nt * kRT + pos) * k;
        for (int e = lane; e < k; e += 32) out[e] = e < c ? sh.L.list[r][e] : kKeyMax;
        if (lane == 0 && sh.L.kth[r] != kKeyMax) atomicMin(&kth_shared[pos], static_cast<unsigned long long>(sh.L.kth[r]));
    }
}

// ---------------------------------------------------------------- merge

// Per row (one warp): the k smallest of the seed list and the S split lists,
// written in the reference's slot order. The lists are sorted, disjoint
// (different columns) and kKeyMax padded, so an element's final rank is its
// position in its own list plus, for every other list, the count of keys
// below it (a binary search in shared memory); no sort is needed. In the
// result the ties with the k-th key already sit at the end in index order;
// the keys below it are placed by counting smaller indices among them.
constexpr int kMergeWarps = 8;

__global__ void __launch_bounds__(32 * kMergeWarps)
merge_kernel(const uint64_t* __restrict__ seed_keys, const uint64_t* __restrict__ partial,
             const unsigned* __restrict__ perm, int64_t n, int nt, int64_t pos0, int64_t pos1, int nsplit, int k,
             int32_t* __restrict__ nbr_idx, float* __restrict__ nbr_d2, float* __restrict__ kdist2) {
    extern __shared__ uint64_t msh[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nl = nsplit + 1, total = nl * k;
    uint64_t* lists = msh + static_cast<int64_t>(warp) * (total + k);
    uint64_t* out = lists + total;
    const int64_t pos = pos0 + static_cast<int64_t>(blockIdx.x) * kMergeWarps + warp;
    if (pos >= pos1) return;
    // element e of the concatenated lists is key t of list l, e = l k + t
    // (found by subtraction: e < (S + 1) k, and division by a run-time k is slow)
    const auto split_index = [k](int e, int& t) {
        int l = 0;
        t = e;
        while (t >= k) {
            t -= k;
            ++l;
        }
        return l;
    };
    for (int e = lane; e < total; e += 32) {
        int t;
        const int l = split_index(e, t);
        lists[e] = (l == 0) ? seed_keys[pos * k + t]
                            : partial[(static_cast<int64_t>(l - 1) * nt * kRT + pos) * k + t];
    }
    for (int e = lane; e < k; e += 32) out[e] = kKeyMax;
    __syncwarp();
    for (int e = lane; e < total; e += 32) {
        const uint64_t x = lists[e];
        if (x == kKeyMax) continue;
        int rank;
        const int l = split_index(e, rank);
        for (int o = 0; o < nl && rank < k; ++o) {
            if (o == l) continue;
            const uint64_t* lo = lists + o * k;
            int a = 0, b = k;  // count of keys < x in list o
            while (a < b) {
                const int mid = (a + b) >> 1;
                if (lo[mid] < x) a = mid + 1;
                else b = mid;
            }
            rank += a;
        }
        if (rank < k) out[rank] = x;
    }
    __syncwarp();
    const uint64_t kth = out[k - 1];
    const uint32_t kbits = key_bits(kth);
    // keys strictly below the k-th occupy out[0, below); the ties follow
    int below = 0;
    for (int e = lane; e < k; e += 32) below += key_bits(out[e]) < kbits ? 1 : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) below += __shfl_xor_sync(0xffffffffu, below, o);
    const unsigned self = perm[pos];
    for (int e = lane; e < k; e += 32) {
        const uint64_t y = out[e];
        int slot = e;  // ties: already in index order after the keys below
        if (e < below) {
            const uint32_t yi = key_index(y);
            slot = 0;
            for (int q = 0; q < below; ++q) slot += key_index(out[q]) < yi ? 1 : 0;
        }
        nbr_idx[static_cast<int64_t>(slot) * n + self] = static_cast<int32_t>(key_index(y) & 0x7FFFFFFFu);
        nbr_d2[static_cast<int64_t>(slot) * n + self] = __uint_as_float(key_bits(y));
    }
    if (lane == 0) kdist2[self] = __uint_as_float(kbits);
}

int grid_for(int64_t items, int block) {
    int64_t g = ceil_div(items, block);
    if (g > 152 * 8) g = 152 * 8;
    return static_cast<int>(g < 1 ? 1 : g);
}

// Whether isolated rows leave the small-d sweep (see iso_rows_kernel):
// from kIsoMinPoints points on (clusters with 1% outliers, d = 8, k = 20,
// fit_predict: 7.72 ms against 8.39 ms at 200,000 points, 3.07 against
// 3.15 at 100,000, 0.82 against 0.92 at 20,000); CULOF_ISO_ROWS=0 or 1
// forces the choice (the results are the same either way).
constexpr int64_t kIsoMinPoints = 16384;
bool iso_rows_enabled(int64_t n) {
    if (const char* env = std::getenv("CULOF_ISO_ROWS")) return env[0] != '0';
    return n >= kIsoMinPoints;
}

}  // namespace

int choose_splits(int nt, int sms) {
    // enough CTAs (2 per SM resident) for ~16 waves, at most 7 splits
    const int want = (32 * sms + nt - 1) / nt;
    int s = want < 1 ? 1 : want;
    if (s > 7) s = 7;
    if (s > nt - 1) s = nt - 1 > 0 ? nt - 1 : 1;
    return s;
}

namespace {

template <int DP, int M>
void launch_sweep(const float* tiles, int nt, int t0, int mt, int qs, int nsplit, int k, const unsigned* maxn,
                  unsigned long long* kth_shared,
                  uint64_t* partial, int* status, unsigned long long* evaluated, const uint2* plist, const int* pcount,
                  const unsigned* order, const float* boxes, const unsigned char* iso_flag, cudaStream_t s) {
    const size_t smem = sizeof(SweepSmem<DP, M>);
    set_max_dynamic_smem(reinterpret_cast<const void*>(sweep_kernel<DP, M>), static_cast<int>(smem));
    sweep_kernel<DP, M><<<mt * nsplit, kThreads, smem, s>>>(tiles, nt, t0, mt, qs, nsplit, k, maxn, kth_shared,
                                                            partial, status, evaluated, plist, pcount, order, boxes,
                                                            iso_flag);
    CG_LAUNCH_CHECK();
}

}  // namespace

void launch_merge(const uint64_t* seed_keys, const uint64_t* partial, const unsigned* perm, int64_t n, int nt,
                  int64_t pos0, int64_t pos1, int nsplit, int k, int32_t* idx, float* d2, float* kd, cudaStream_t s) {
    const size_t smem = sizeof(uint64_t) * kMergeWarps * static_cast<size_t>((nsplit + 1) * k + k);
    if (smem > 48 * 1024)
        CG_CUDA(cudaFuncSetAttribute(merge_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    if (pos1 <= pos0) return;
    merge_kernel<<<static_cast<unsigned>(ceil_div(pos1 - pos0, kMergeWarps)), 32 * kMergeWarps, smem, s>>>(
        seed_keys, partial, perm, n, nt, pos0, pos1, nsplit, k, idx, d2, kd);
    CG_LAUNCH_CHECK();
}

size_t sort_pairs_counts(int64_t n) { return static_cast<size_t>(256) * static_cast<size_t>(ceil_div(n, kSortTile)); }

unsigned* sort_pairs_stable(unsigned* keys, unsigned* vals, unsigned* keys_tmp, unsigned* vals_tmp, int64_t n,
                            int key_bits, unsigned* counts, cudaStream_t s, unsigned** vals_out) {
    const int nblocks = static_cast<int>(ceil_div(n, kSortTile));
    unsigned *kin = keys, *vin = vals, *kout = keys_tmp, *vout = vals_tmp;
    for (int shift = 0; shift < key_bits; shift += 8) {
        sort_upsweep_kernel<<<nblocks, kSortThreads, 0, s>>>(kin, n, shift, counts, nblocks);
        CG_LAUNCH_CHECK();
        sort_scan_kernel<<<1, 1024, 0, s>>>(counts, static_cast<int64_t>(256) * nblocks);
        CG_LAUNCH_CHECK();
        sort_downsweep_kernel<<<nblocks, kSortThreads, 0, s>>>(kin, vin, kout, vout, n, shift, counts, nblocks);
        CG_LAUNCH_CHECK();
        unsigned* t = kin;
        kin = kout;
        kout = t;
        t = vin;
        vin = vout;
        vout = t;
    }
    *vals_out = vin;
    return kin;
}

void exclusive_scan_u32(unsigned* data, int64_t len, cudaStream_t s) {
    sort_scan_kernel<<<1, 1024, 0, s>>>(data, len);
    CG_LAUNCH_CHECK();
}

bool fast_path_supported(int64_t n, int d, int k) {
    return d >= 1 && d <= kMaxWideD && k >= 1 && k <= kMaxK && n >= 2 && static_cast<int64_t>(k) < n &&
           n <= (static_cast<int64_t>(1) << 30);
}

// Host orchestration of the fast path.
void Engine::knn_fast(const float* xc, const float* norms, int64_t n, int d, int k, bool tensor, int32_t* nbr_idx,
                      float* nbr_d2, float* kdist2, int shard, int num_shards, int32_t* shard_rows) {
    cudaStream_t s = stream_;
    const bool wide = !tensor && d > kMaxDP;
    // the tensor sweep for d <= 8 starts from the small-d seed window and
    // visits only the column tiles of the small-d prune lists
    const bool small_tc = tensor && d <= kMaxDP;
    const bool small = !wide && (!tensor || small_tc);  // FP32 small-d tiles, boxes and seed
    const int dp = d <= 2 ? 2 : d <= 4 ? 4 : d <= 6 ? 6 : 8;
    const int nt = static_cast<int>(ceil_div(n, kCT));
    const int64_t padded = static_cast<int64_t>(nt) * kCT;
    // the rows of this call: row tiles [t0, t0 + mt) of the spatial order
    // (all of them unless the call is one shard of a row-sharded run)
    const int t0 = static_cast<int>(static_cast<int64_t>(nt) * shard / num_shards);
    const int mt = static_cast<int>(static_cast<int64_t>(nt) * (shard + 1) / num_shards) - t0;
    int sms = 152;
    CG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    // The tensor sweep runs two CTAs per SM. Every split of a row tile starts
    // from the loose seed threshold and pays the candidate surge that follows,
    // so it takes few splits: one from two waves of row tiles up, otherwise
    // enough for about 4 x SMs CTAs (two waves at two per SM), at most 3
    // (measured on 20k-50k point clusters in 32-128 dimensions: 3.9-9.6 ms
    // against 5.0-11.5 ms with 7).
    int nsplit = 1;
    if (nt > 1) {
        if (wide) {
            nsplit = choose_splits(mt, sms);
            if (nsplit > nt - 1) nsplit = nt - 1;
        } else if (!tensor) {
            // small-d sweep: about 9 waves of CTAs (2 per SM); more splits
            // only add merge work and restart more rows from the seed, fewer
            // leave the tail unbalanced (measured best: 7 splits at n = 50k,
            // 3 at 100k (3.33 ms against 3.73 ms with 7), 2 at 200k (8.85 ms
            // against 9.15 ms with 4))
            nsplit = mt > 0 ? (18 * sms + mt / 2) / mt : 1;
            nsplit = nsplit < 1 ? 1 : nsplit > 7 ? 7 : nsplit;
        } else if (mt < 4 * sms) {
            nsplit = mt > 0 ? (4 * sms + mt / 2) / mt : 1;
            nsplit = nsplit < 1 ? 1 : nsplit > 3 ? 3 : nsplit;
            if (nsplit > nt - 1) nsplit = nt - 1;
        }
    }
    if (const char* env = std::getenv("CULOF_SPLITS")) {  // tuning override (1..nt-1)
        const long v = std::atol(env);
        if (v >= 1 && nt > 1) nsplit = static_cast<int>(v < nt - 1 ? v : nt - 1);
    }
    // the small-d seed covers the first qs spiral positions of every row
    // tile, the sweep the rest (the wide and tensor seeds cover tile T alone)
    const int qs = small ? (nt < kSeedWindow ? nt : kSeedWindow) : 1;
    const bool sweep = nt > qs;
    if (sweep && nsplit > nt - qs) nsplit = nt - qs;  // no split without a column tile

    // 1. Morton keys of the centred coordinates, then a stable radix sort.
    unsigned* mm = reinterpret_cast<unsigned*>(sort_hist_.get(2 * sizeof(unsigned) * d + sizeof(int) * kMortonDims));
    int* dims = reinterpret_cast<int*>(mm + 2 * d);
    unsigned* keys = morton_.as<unsigned>(2 * static_cast<size_t>(n));
    unsigned* vals = perm_.as<unsigned>(2 * static_cast<size_t>(n));
    minmax_init_kernel<<<1, 32, 0, s>>>(mm, d);
    CG_LAUNCH_CHECK();
    minmax_kernel<<<grid_for(n * d, 256), 256, 0, s>>>(xc, n, d, mm);
    CG_LAUNCH_CHECK();
    select_dims_kernel<<<1, 32, 0, s>>>(mm, d, dims);
    CG_LAUNCH_CHECK();
    morton_kernel<<<grid_for(n, 256), 256, 0, s>>>(xc, n, d, mm, dims, keys, vals);
    CG_LAUNCH_CHECK();
    const int nblocks = static_cast<int>(ceil_div(n, kSortTile));
    unsigned* counts = sort_tmp_.as<unsigned>(static_cast<size_t>(256) * nblocks);
    unsigned *kin = keys, *vin = vals, *kout = keys + n, *vout = vals + n;
    for (int pass = 0; pass < 4; ++pass) {
        const int shift = 8 * pass;
        sort_upsweep_kernel<<<nblocks, kSortThreads, 0, s>>>(kin, n, shift, counts, nblocks);
        CG_LAUNCH_CHECK();
        sort_scan_kernel<<<1, 1024, 0, s>>>(counts, static_cast<int64_t>(256) * nblocks);
        CG_LAUNCH_CHECK();
        sort_downsweep_kernel<<<nblocks, kSortThreads, 0, s>>>(kin, vin, kout, vout, n, shift, counts, nblocks);
        CG_LAUNCH_CHECK();
        unsigned* t = kin;
        kin = kout;
        kout = t;
        t = vin;
        vin = vout;
        vout = t;
    }
    const unsigned* perm = vin;  // after 4 passes: back in the first half
    const int64_t pos0 = static_cast<int64_t>(t0) * kCT;
    const int64_t pos1 = std::min<int64_t>(n, static_cast<int64_t>(t0 + mt) * kCT);
    if (shard_rows && pos1 > pos0)  // original indices of the shard's rows
        CG_CUDA(cudaMemcpyAsync(shard_rows, perm + pos0, sizeof(unsigned) * (pos1 - pos0), cudaMemcpyDeviceToDevice,
                                s));

    // 2. column tiles
    float* tiles = nullptr;
    TcBuffers tcb{};
    float* boxes = nullptr;
    if (tensor) tcb = tc_prepare(cols_.get(tc_buffer_bytes(padded, d)), xc, norms, n, d, perm, nt, mm, s);
    DevBuf& small_tiles = small_tc ? tiles_ : cols_;
    if (wide) {
        tiles = cols_.as<float>(wide_tiles_floats(d, nt));
        wide_build_tiles(xc, norms, n, d, perm, nt, tiles, s);
    } else if (small) switch (dp) {
        case 2: tiles = small_tiles.as<float>(static_cast<size_t>(tile_floats(2)) * nt); break;
        case 4: tiles = small_tiles.as<float>(static_cast<size_t>(tile_floats(4)) * nt); break;
        case 6: tiles = small_tiles.as<float>(static_cast<size_t>(tile_floats(6)) * nt); break;
        default: tiles = small_tiles.as<float>(static_cast<size_t>(tile_floats(8)) * nt); break;
    }
    if (small) switch (dp) {
        case 2: build_tiles_kernel<2><<<grid_for(padded, 256), 256, 0, s>>>(xc, norms, n, d, perm, padded, tiles); break;
        case 4: build_tiles_kernel<4><<<grid_for(padded, 256), 256, 0, s>>>(xc, norms, n, d, perm, padded, tiles); break;
        case 6: build_tiles_kernel<6><<<grid_for(padded, 256), 256, 0, s>>>(xc, norms, n, d, perm, padded, tiles); break;
        default: build_tiles_kernel<8><<<grid_for(padded, 256), 256, 0, s>>>(xc, norms, n, d, perm, padded, tiles); break;
    }
    if (small) {
        CG_LAUNCH_CHECK();
        boxes = boxes_.as<float>(static_cast<size_t>(nt) * 2 * dp);
        const unsigned bg = static_cast<unsigned>(ceil_div(nt, 8));
        switch (dp) {
            case 2: tile_box_kernel<2><<<bg, 256, 0, s>>>(tiles, nt, boxes); break;
            case 4: tile_box_kernel<4><<<bg, 256, 0, s>>>(tiles, nt, boxes); break;
            case 6: tile_box_kernel<6><<<bg, 256, 0, s>>>(tiles, nt, boxes); break;
            default: tile_box_kernel<8><<<bg, 256, 0, s>>>(tiles, nt, boxes); break;
        }
        CG_LAUNCH_CHECK();
    }

    // 3. seed lists and the shared k-th keys
    char* rows = static_cast<char*>(rows_.get(padded * sizeof(uint64_t) * (k + 1) +
                                              static_cast<size_t>(nsplit) * padded * k * sizeof(uint64_t) + 256));
    uint64_t* seed_keys = reinterpret_cast<uint64_t*>(rows);
    unsigned long long* kth_shared = reinterpret_cast<unsigned long long*>(seed_keys + padded * k);
    uint64_t* partial = reinterpret_cast<uint64_t*>(kth_shared + padded);
    int* status = status_ptr();
    const unsigned* maxn = reinterpret_cast<const unsigned*>(max_norm_.get(sizeof(unsigned)));
    mark(2);
    if (tensor && !small_tc) tc_seed(tcb, t0, mt, d, k, seed_keys, kth_shared, s);
    else if (wide) wide_seed(tiles, nt, t0, mt, d, k, seed_keys, kth_shared, s);
    else switch (dp) {
        case 2: seed_kernel<2><<<mt, kThreads, 0, s>>>(tiles, nt, t0, n, k, qs, seed_keys, kth_shared); break;
        case 4: seed_kernel<4><<<mt, kThreads, 0, s>>>(tiles, nt, t0, n, k, qs, seed_keys, kth_shared); break;
        case 6: seed_kernel<6><<<mt, kThreads, 0, s>>>(tiles, nt, t0, n, k, qs, seed_keys, kth_shared); break;
        default: seed_kernel<8><<<mt, kThreads, 0, s>>>(tiles, nt, t0, n, k, qs, seed_keys, kth_shared); break;
    }
    if (small) CG_LAUNCH_CHECK();
    mark(3);

    // 3a. isolated rows (the FP32 small-d sweep): about 1% of the rows, those
    // with the largest seed k-th keys, leave the sweep for their own pass
    unsigned char* iso_flag = nullptr;
    int* iso_list = nullptr;
    int* iso_count = nullptr;
    const int64_t pend = static_cast<int64_t>(t0 + mt) * kCT;
    // at most about 2% of the rows (a sample threshold that ties with many
    // equal k-th keys could otherwise take far more than 1%)
    const int iso_cap = static_cast<int>((pos1 - pos0) / 50 + 32);
    if (small && !tensor && sweep && mt > 0 && pos1 > pos0 && nt <= kIsoMaxTiles && iso_rows_enabled(n)) {
        char* b = static_cast<char*>(
            iso_.get(256 + sizeof(int) * static_cast<size_t>(pend - pos0) + padded + 256 + sizeof(unsigned) * kIsoBins));
        unsigned long long* thr = reinterpret_cast<unsigned long long*>(b);
        iso_count = reinterpret_cast<int*>(b + sizeof(unsigned long long));
        iso_list = reinterpret_cast<int*>(b + 256);
        iso_flag = reinterpret_cast<unsigned char*>(iso_list + (pend - pos0));  // indexed by position
        unsigned* hist = reinterpret_cast<unsigned*>(b + 256 + sizeof(int) * static_cast<size_t>(pend - pos0) + padded);
        CG_CUDA(cudaMemsetAsync(hist, 0, sizeof(unsigned) * kIsoBins, s));
        iso_hist_kernel<<<grid_for(pos1 - pos0, 256), 256, 0, s>>>(kth_shared, pos0, pos1, hist);
        CG_LAUNCH_CHECK();
        iso_threshold_kernel<<<1, 1024, 0, s>>>(hist, pos1 - pos0, thr, iso_count);
        CG_LAUNCH_CHECK();
        iso_mark_kernel<<<grid_for(pend - pos0, 256), 256, 0, s>>>(kth_shared, pos0, pend, n, thr, iso_cap, iso_flag,
                                                                   iso_list, iso_count);
        CG_LAUNCH_CHECK();
    }

    // 3b. per row tile: the column tiles the seed's k-th distances leave
    uint2* plist = nullptr;
    int* pcount = nullptr;
    const unsigned* order = nullptr;
    constexpr int kMaxListTiles = 16384;  // lists take nt^2 x 8 bytes: up to 2 GiB
    // CULOF_PRUNE_LISTS=0 walks the whole spiral as inputs above the list
    // limit do (the same results; it puts that path within reach of tests)
    const char* lists_env = std::getenv("CULOF_PRUNE_LISTS");
    const bool lists_on = !(lists_env && lists_env[0] == '0');
    if (small && sweep && nt <= kMaxListTiles && lists_on) {
        plist = plist_.as<uint2>(static_cast<size_t>(nt) * nt);
        pcount = pcount_.as<int>(nt);
        switch (dp) {
            case 2: prune_list_kernel<2><<<mt, 256, 0, s>>>(boxes, nt, t0, qs, kth_shared, plist, pcount, tiles, iso_flag); break;
            case 4: prune_list_kernel<4><<<mt, 256, 0, s>>>(boxes, nt, t0, qs, kth_shared, plist, pcount, tiles, iso_flag); break;
            case 6: prune_list_kernel<6><<<mt, 256, 0, s>>>(boxes, nt, t0, qs, kth_shared, plist, pcount, tiles, iso_flag); break;
            default: prune_list_kernel<8><<<mt, 256, 0, s>>>(boxes, nt, t0, qs, kth_shared, plist, pcount, tiles, iso_flag); break;
        }
        CG_LAUNCH_CHECK();
    }
    // launch order: longest lists first (balances the tail of a many-wave
    // grid; small grids skip the sort)
    if (plist && !tensor && mt >= 4 * sms) {
        unsigned* ok = reinterpret_cast<unsigned*>(order_.get(sizeof(unsigned) * (4 * static_cast<size_t>(mt) +
                                                                                   sort_pairs_counts(mt))));
        order_key_kernel<<<grid_for(mt, 256), 256, 0, s>>>(pcount, t0, mt, ok, ok + mt);
        CG_LAUNCH_CHECK();
        unsigned* sorted_vals = nullptr;
        sort_pairs_stable(ok, ok + mt, ok + 2 * mt, ok + 3 * mt, mt, 16, ok + 4 * mt, s, &sorted_vals);
        order = sorted_vals;
    }

    // 4. sweep over the other tiles, split S ways
    unsigned long long* evaluated = reinterpret_cast<unsigned long long*>(pair_stats_.get(2 * sizeof(unsigned long long)));
    CG_CUDA(cudaMemsetAsync(evaluated, 0, 2 * sizeof(unsigned long long), s));
    // With isolated rows, the sweep and their pass become ready together on
    // two forked streams, the sweep's of higher priority: its CTAs are
    // dispatched first and the pass fills the SMs its last wave leaves.
    cudaStream_t sweep_s = s;
    if (iso_flag) {
        make_fork_streams();
        CG_CUDA(cudaEventRecord(fork_ev_, s));
        CG_CUDA(cudaStreamWaitEvent(high_stream_, fork_ev_, 0));
        sweep_s = high_stream_;
    }
    // every (warp, column tile) block past the seed window
    stat_total_blocks_ = (small && !tensor && sweep) ? static_cast<unsigned long long>(mt) * (nt - qs) * kWarps : 0;
    if (sweep && mt > 0 && tensor) {
        uint64_t* lists = static_cast<uint64_t*>(tc_lists_.get(tc_list_bytes(mt, nsplit)));
        tc_sweep(tcb, nt, t0, mt, nsplit, d, k, maxn, kth_shared, partial, lists, status, s, qs, plist, pcount);
    } else if (nt > 1 && mt > 0 && wide) {
        wide_sweep(tiles, nt, t0, mt, nsplit, d, k, maxn, kth_shared, partial, s);
    } else if (sweep && mt > 0) {
        // lists of 64 keys for k <= 24, 96 for k <= 48, else 128: a list
        // compacts once fewer than 32 slots are free, so k close to the
        // capacity minus 32 would compact after every chunk (k = 32 with 64
        // slots: 1.90 ms against 1.44 ms for k = 33 with 96, n = 20k; k = 64
        // with 96 slots: 42.1 ms at n = 200k, against 21.1 ms for k = 56).
        // Above 64 slots a CTA per SM is what the shared memory allows
        // anyway.
#define CG_SWEEP_M(DPV, MV)                                                                                           \
    launch_sweep<DPV, MV>(tiles, nt, t0, mt, qs, nsplit, k, maxn, kth_shared, partial, status, evaluated, plist, pcount, \
                          order, boxes, iso_flag, sweep_s)
#define CG_SWEEP(DPV) (k > 48 ? CG_SWEEP_M(DPV, 128) : k > 24 ? CG_SWEEP_M(DPV, 96) : CG_SWEEP_M(DPV, 64))
        switch (dp) {
            case 2: CG_SWEEP(2); break;
            case 4: CG_SWEEP(4); break;
            case 6: CG_SWEEP(6); break;
            default: CG_SWEEP(8); break;
        }
#undef CG_SWEEP
#undef CG_SWEEP_M
    }
    if (iso_flag) {  // the isolated rows' own pass (split-0 lists), on the side stream
        CG_CUDA(cudaEventRecord(high_join_, high_stream_));
        CG_CUDA(cudaStreamWaitEvent(s, high_join_, 0));
        cudaStream_t side = side_stream_;
        CG_CUDA(cudaStreamWaitEvent(side, fork_ev_, 0));
        const int g = 6 * sms;  // one CTA per row, grid-stride (six CTAs per SM)
        const size_t qgap_bytes = sizeof(uint16_t) * kQuarters * static_cast<size_t>(nt);
        // columns (nt x kCT x dp floats), then the quarter boxes (32 bytes each)
        float* cols = iso_cols_.as<float>(static_cast<size_t>(nt) * (kCT * dp + kQuarters * 8));
        __nv_bfloat16* qbox = reinterpret_cast<__nv_bfloat16*>(cols + static_cast<size_t>(nt) * kCT * dp);
        constexpr size_t kDefaultDynamicSmem = 40 * 1024;
#define CG_ISO(DPV)                                                                                                \
    iso_cols_kernel<DPV><<<grid_for(static_cast<int64_t>(nt) * DPV * kCT, 256), 256, 0, side>>>(tiles, nt, cols);   \
    CG_LAUNCH_CHECK();                                                                                             \
    iso_qbox_kernel<DPV><<<grid_for(static_cast<int64_t>(nt) * kQuarters * 32, 256), 256, 0, side>>>(tiles, cols, nt, \
                                                                                                   qbox);          \
    CG_LAUNCH_CHECK();                                                                                             \
    if (qgap_bytes > kDefaultDynamicSmem)                                                                          \
        set_max_dynamic_smem(reinterpret_cast<const void*>(iso_rows_kernel<DPV>), static_cast<int>(qgap_bytes));  \
    iso_rows_kernel<DPV><<<g, 32 * kIsoWarps, qgap_bytes, side>>>(tiles, cols, qbox, nt, qs, k, iso_cap, iso_list,    \
                                                               iso_count, kth_shared, partial)
        switch (dp) {
            case 2: CG_ISO(2); break;
            case 4: CG_ISO(4); break;
            case 6: CG_ISO(6); break;
            default: CG_ISO(8); break;
        }
#undef CG_ISO
        CG_LAUNCH_CHECK();
        CG_CUDA(cudaEventRecord(side_join_, side));
        CG_CUDA(cudaStreamWaitEvent(s, side_join_, 0));
    }
    const int ns = sweep ? nsplit : 0;
    mark(4);

    // 5. merge into the reference slot order
    launch_merge(seed_keys, partial, perm, n, nt, pos0, pos1, ns, k, nbr_idx, nbr_d2, kdist2, s);
}

}  // namespace culof_gb300
