// General exact k-NN path: an exact-distance tile (rows x n) written to HBM,
// then an exact per-row select over it. It serves any k in [1, n-1] and any
// d, and it is the engine's implementation of the reference's internal tile
// contract (culof_internal.cuh:37-53: select_knn over a Gram tile), which the
// tests drive with injected distances.
//
// Rules kept from the reference (the outputs must be the same bits):
//   * key = IEEE bits of the non-negative squared distance, ordered as uint32;
//     the k-distance is the float of the k-th smallest key (knn.cu:180-184);
//   * slot order: every key strictly below the k-th in ascending column
//     index, then the keys equal to it in ascending column index until k
//     slots are filled (knn.cu:190-224);
//   * outputs are transposed: slot t of point i at [t * n + i];
//   * in kSelectGram mode a Gram value g becomes
//     max(0, (|x_self|^2 + |x_j|^2) - 2 g), +inf for the diagonal and NaN,
//     stored back in place (knn.cu:150-152); in kSelectDistances mode the
//     tile already holds exact distances and the diagonal is skipped.
// The select itself (row_select_kernel below) is this engine's own design.
#include "block.cuh"
#include "common.cuh"
#include "prep.cuh"
#include "warp_sort.cuh"

namespace culof_gb300 {

namespace {

constexpr int kTileBlock = 256;   // columns per block of the distance tile
constexpr int kTileRows = 16;     // rows per block of the distance tile
constexpr int kTileDimChunk = 32; // dims staged per step

// tile[r * n + j] = dist2_direct(xc[row0 + r], xc[j]) for r < rows, j < n.
// Dims are accumulated chunk by chunk in ascending order with the running sum
// carried across chunks, which is exactly dist2_direct's operation order.
__global__ void __launch_bounds__(kTileBlock)
distance_tile_kernel(const float* __restrict__ xc, int64_t n, int d, int64_t row0, int rows,
                     float* __restrict__ tile) {
    __shared__ float srow[kTileRows][kTileDimChunk];
    __shared__ float scol[kTileBlock][kTileDimChunk + 1];
    const int64_t col0 = static_cast<int64_t>(blockIdx.x) * kTileBlock;
    const int r0 = blockIdx.y * kTileRows;
    const int tid = threadIdx.x;
    float acc[kTileRows];
#pragma unroll
    for (int r = 0; r < kTileRows; ++r) acc[r] = 0.0f;

    for (int f0 = 0; f0 < d; f0 += kTileDimChunk) {
        const int df = min(kTileDimChunk, d - f0);
        for (int e = tid; e < kTileRows * kTileDimChunk; e += kTileBlock) {
            const int r = e / kTileDimChunk, f = e % kTileDimChunk;
            float v = 0.0f;
            if (r0 + r < rows && f < df) v = xc[(row0 + r0 + r) * d + f0 + f];
            srow[r][f] = v;
        }
        for (int e = tid; e < kTileBlock * kTileDimChunk; e += kTileBlock) {
            const int c = e / kTileDimChunk, f = e % kTileDimChunk;
            float v = 0.0f;
            if (col0 + c < n && f < df) v = xc[(col0 + c) * d + f0 + f];
            scol[c][f] = v;
        }
        __syncthreads();
        for (int f = 0; f < df; ++f) {
            const float b = scol[tid][f];
#pragma unroll
            for (int r = 0; r < kTileRows; ++r) {
                const float t = __fsub_rn(srow[r][f], b);
                acc[r] = __fmaf_rn(t, t, acc[r]);
            }
        }
        __syncthreads();
    }
    const int64_t j = col0 + tid;
    if (j < n) {
#pragma unroll
        for (int r = 0; r < kTileRows; ++r)
            if (r0 + r < rows) tile[static_cast<int64_t>(r0 + r) * n + j] = acc[r];
    }
}

// ---------------------------------------------------------------- row select
//
// One CTA per row selects the row's k smallest keys (the IEEE bits of the
// non-negative squared distance, ties by column index) and writes them in
// slot order. The design:
//   * each warp owns one contiguous segment of the row's columns and walks
//     it 32 columns at a time, so every pass is coalesced and every loop is
//     warp-uniform;
//   * a 4096-bin histogram of the keys' bits 30..19 (bit 31 is always 0)
//     built with warp-aggregated shared atomics (lanes with the same bin
//     elect one adder) locates the bucket of the k-th key; a warp narrows the
//     bins by ballots over lane prefix sums (4096 -> 128 -> 4 -> 1);
//   * the keys of that bucket (typically a few dozen) are copied to shared
//     memory with their columns and sorted, which gives the k-th key: up to
//     128 keys by one warp in registers (no block barrier), more by the whole
//     block (bitonic in shared memory); a bucket too large for the buffer is
//     narrowed first by a second
//     histogram (bits 18..7) and, if still too large, by a third (bits 6..0),
//     which pins the k-th key's bits exactly;
//   * every warp knows how many keys of its segment lie below the k-th key
//     and how many equal it (from the extraction pass and the sorted bucket),
//     so a warp-level exclusive scan gives each segment its first slot, and
//     the emission pass ranks keys inside a 32-column step with ballots:
//     keys below the k-th in ascending column order fill slots [0, below),
//     keys equal to it fill [below, k) in ascending column order.
// Rows of up to kRowCache keys stay in shared memory after the first pass.

constexpr int kSelThreads = 256;
constexpr int kSelWarps = kSelThreads / 32;
constexpr int kBins = 4096;
constexpr int kCandCap = 2048;
constexpr int kRowCache = 4096;
constexpr unsigned kFull = 0xffffffffu;

struct RowSelect {
    int hist[kBins];
    unsigned long long cand[kCandCap];  // (key << 32) | column of the k-th key's bucket
    int warp_lt[kSelWarps];             // keys of each warp's segment below the k-th key
    int warp_eq[kSelWarps];             // keys equal to it
    int ncand;
    unsigned prefix;  // high bits of the k-th key found so far
    int below;        // keys strictly below the current bucket
    int need;         // rank of the k-th key inside the current bucket (1-based)
    int bucket;       // keys inside the current bucket
    unsigned kth;     // the k-th key, once found
};

// Levels of the bucket search: (lowest bit, width). Keys are < 2^31.
__device__ __forceinline__ int level_shift(int lv) { return lv == 0 ? 19 : (lv == 1 ? 7 : 0); }
__device__ __forceinline__ int level_width(int lv) { return lv == 2 ? 7 : 12; }

// Adds 1 to hist[bin] for every lane with `take`; lanes that share a bin
// elect one adder. All 32 lanes must call it.
__device__ __forceinline__ void hist_add(int* hist, unsigned bin, bool take) {
    const unsigned active = __ballot_sync(kFull, take);
    if (!take) return;
    const unsigned peers = __match_any_sync(active, bin);
    if ((threadIdx.x & 31) == __ffs(peers) - 1) atomicAdd(&hist[bin], __popc(peers));
}

// One warp: the bin holding the need-th key (1-based) of a histogram of
// `bins` = 32 * 4^m entries. Each round splits the remaining range into 32
// equal parts, one per lane, and keeps the part where the lanes' inclusive
// prefix sums first reach `need` (a ballot). Returns the bin and sets the
// keys below it and the keys inside it.
__device__ int locate_bin(const int* hist, int bins, int need, int& below, int& inside) {
    const int lane = threadIdx.x & 31;
    int base = 0, span = bins, acc = 0;
    while (true) {
        const int part = span / 32 > 0 ? span / 32 : 1;
        int s = 0;
        if (lane * part < span)
            for (int i = 0; i < part; ++i) s += hist[base + lane * part + i];
        const int incl = warp_inclusive_scan(s);
        const unsigned hit = __ballot_sync(kFull, acc + incl >= need);
        const int L = hit ? __ffs(hit) - 1 : 31;  // counts are consistent: hit != 0
        const int excl = __shfl_sync(kFull, incl - s, L);
        const int own = __shfl_sync(kFull, s, L);
        acc += excl;
        base += L * part;
        if (part == 1) {
            below = acc;
            inside = own;
            return base;
        }
        span = part;
    }
}

// Column j of the row as a key, from the shared-memory copy when the row
// fits there.
__device__ __forceinline__ unsigned row_key(const float* row, const unsigned* cache, bool cached, int64_t j) {
    return cached ? cache[j] : __float_as_uint(row[j]);
}

__global__ void __launch_bounds__(kSelThreads)
row_select_kernel(float* __restrict__ tile, const float* __restrict__ norms, int rows, int64_t row_offset,
                  int64_t n, int k, int mode, int32_t* __restrict__ nbr_idx, float* __restrict__ nbr_d2,
                  float* __restrict__ kdist2) {
    __shared__ RowSelect sh;
    extern __shared__ unsigned cache[];
    const int r = blockIdx.x;
    if (r >= rows) return;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool gram = (mode == kSelectGram);
    const bool cached = n <= kRowCache;
    float* row = tile + static_cast<int64_t>(r) * n;
    const int64_t self = row_offset + r;
    // warp segments: contiguous, a multiple of 32 columns each
    const int64_t seg = ceil_div(ceil_div(n, kSelWarps), 32) * 32;
    const int64_t s0 = static_cast<int64_t>(warp) * seg;
    const int64_t s1 = s0 + seg < n ? s0 + seg : n;

    for (int b = threadIdx.x; b < kBins; b += kSelThreads) sh.hist[b] = 0;
    if (threadIdx.x == 0) {
        sh.prefix = 0u;
        sh.below = 0;
        sh.need = k;
    }
    __syncthreads();

    // level 0 histogram (and the Gram conversion, written back in place)
    const float self_norm = gram ? norms[self] : 0.0f;
    for (int64_t j0 = s0; j0 < s1; j0 += 32) {
        const int64_t j = j0 + lane;
        const bool in = j < s1;
        unsigned u = 0;
        if (in) {
            if (gram) {
                const float raw = __fsub_rn(__fadd_rn(self_norm, norms[j]), __fmul_rn(2.0f, row[j]));
                const float d2 = (j == self || isnan(raw)) ? __int_as_float(0x7f800000) : fmaxf(0.0f, raw);
                row[j] = d2;
                u = __float_as_uint(d2);
            } else {
                u = __float_as_uint(row[j]);
            }
            if (cached) cache[j] = u;
        }
        // a point is never its own neighbour in distance mode; in Gram mode
        // the diagonal is +inf and takes part, as the reference contract has it
        hist_add(sh.hist, (u >> 19) & (kBins - 1), in && (gram || j != self));
    }
    __syncthreads();

    int level = 0;
    while (true) {
        if (warp == 0) {
            int below = 0, inside = 0;
            const int bin = locate_bin(sh.hist, 1 << level_width(level), sh.need, below, inside);
            if (lane == 0) {
                sh.prefix |= static_cast<unsigned>(bin) << level_shift(level);
                sh.below += below;
                sh.need -= below;
                sh.bucket = inside;
                sh.ncand = 0;
            }
        }
        __syncthreads();
        if (sh.bucket <= kCandCap || level == 2) break;
        // narrow the bucket with the next digit
        ++level;
        const int shift = level_shift(level);
        const int hi = shift + level_width(level);
        const unsigned want = sh.prefix >> hi;
        for (int b = threadIdx.x; b < (1 << level_width(level)); b += kSelThreads) sh.hist[b] = 0;
        __syncthreads();
        for (int64_t j0 = s0; j0 < s1; j0 += 32) {
            const int64_t j = j0 + lane;
            const bool in = j < s1 && (gram || j != self);
            const unsigned u = in ? row_key(row, cache, cached, j) : 0u;
            hist_add(sh.hist, (u >> shift) & ((1u << level_width(level)) - 1u), in && (u >> hi) == want);
        }
        __syncthreads();
    }

    const int shift = level_shift(level);
    const unsigned want = sh.prefix >> shift;
    unsigned kth;
    if (level == 2 && sh.bucket > kCandCap) {
        // every key of the final bucket has the same bits: the k-th key
        kth = sh.prefix;
        int lt = 0, eq = 0;
        for (int64_t j0 = s0; j0 < s1; j0 += 32) {
            const int64_t j = j0 + lane;
            const bool in = j < s1 && (gram || j != self);
            const unsigned u = in ? row_key(row, cache, cached, j) : 0u;
            lt += __popc(__ballot_sync(kFull, in && u < kth));
            eq += __popc(__ballot_sync(kFull, in && u == kth));
        }
        if (lane == 0) {
            sh.warp_lt[warp] = lt;
            sh.warp_eq[warp] = eq;
        }
        __syncthreads();
    } else {
        // copy the bucket's keys with their columns; count the keys below it
        int lt = 0;
        for (int64_t j0 = s0; j0 < s1; j0 += 32) {
            const int64_t j = j0 + lane;
            const bool in = j < s1 && (gram || j != self);
            const unsigned u = in ? row_key(row, cache, cached, j) : 0u;
            const bool take = in && (u >> shift) == want;
            lt += __popc(__ballot_sync(kFull, in && (u >> shift) < want));
            const unsigned m = __ballot_sync(kFull, take);
            int slot0 = 0;
            if (lane == 0 && m) slot0 = atomicAdd(&sh.ncand, __popc(m));
            slot0 = __shfl_sync(kFull, slot0, 0);
            const int slot = slot0 + __popc(m & ((1u << lane) - 1u));
            if (take && slot < kCandCap)
                sh.cand[slot] = (static_cast<unsigned long long>(u) << 32) | static_cast<unsigned long long>(j);
        }
        if (lane == 0) {
            sh.warp_lt[warp] = lt;
            sh.warp_eq[warp] = 0;
        }
        __syncthreads();
        const int m = sh.ncand;
        if (m <= 128) {
            // the usual case: one warp sorts the bucket in registers (a
            // 128-key bitonic network, element e = lane + 32 j) and counts
            // its keys below / equal to the k-th by owning warp; no block
            // barrier until the result is published
            if (warp == 0) {
                uint64_t v[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int e = 32 * j + lane;
                    v[j] = e < m ? sh.cand[e] : ~0ull;
                }
                warp_bitonic_sort<4>(v);
                const int rk = sh.need - 1;
                uint64_t kk = 0;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const uint64_t t = __shfl_sync(kFull, v[j], rk & 31);
                    if (j == (rk >> 5)) kk = t;
                }
                const unsigned kb = static_cast<unsigned>(kk >> 32);
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (32 * j + lane < m) {
                        const unsigned u = static_cast<unsigned>(v[j] >> 32);
                        const int w = static_cast<int>(static_cast<int64_t>(v[j] & 0xffffffffull) / seg);
                        if (u < kb) atomicAdd(&sh.warp_lt[w], 1);
                        else if (u == kb) atomicAdd(&sh.warp_eq[w], 1);
                    }
                }
                if (lane == 0) sh.kth = kb;
            }
            __syncthreads();
            kth = sh.kth;
        } else {
        // bitonic sort of the bucket, padded to a power of two with ~0
        int len = 1;
        while (len < m) len <<= 1;
        for (int i = m + threadIdx.x; i < len; i += kSelThreads) sh.cand[i] = ~0ull;
        __syncthreads();
        for (int size = 2; size <= len; size <<= 1) {
            for (int stride = size >> 1; stride > 0; stride >>= 1) {
                for (int i = threadIdx.x; i < len / 2; i += kSelThreads) {
                    const int lo = 2 * i - (i & (stride - 1));
                    const int hi2 = lo + stride;
                    const bool up = (lo & size) == 0;
                    const unsigned long long a = sh.cand[lo], b = sh.cand[hi2];
                    if ((a > b) == up) {
                        sh.cand[lo] = b;
                        sh.cand[hi2] = a;
                    }
                }
                __syncthreads();
            }
        }
        kth = static_cast<unsigned>(sh.cand[sh.need - 1] >> 32);
        // the bucket's keys below / equal to the k-th key, by owning warp
        for (int i = threadIdx.x; i < m; i += kSelThreads) {
            const unsigned u = static_cast<unsigned>(sh.cand[i] >> 32);
            const int w = static_cast<int>(static_cast<int64_t>(sh.cand[i] & 0xffffffffull) / seg);
            if (u < kth) atomicAdd(&sh.warp_lt[w], 1);
            else if (u == kth) atomicAdd(&sh.warp_eq[w], 1);
        }
        __syncthreads();
        }
    }

    // first slot of each segment: exclusive scans over the warps' counts
    int lt_base = 0, eq_base = 0, below_all = 0;
    {
        const int my_lt = lane < kSelWarps ? sh.warp_lt[lane] : 0;
        const int my_eq = lane < kSelWarps ? sh.warp_eq[lane] : 0;
        const int lt_incl = warp_inclusive_scan(my_lt);
        const int eq_incl = warp_inclusive_scan(my_eq);
        lt_base = __shfl_sync(kFull, lt_incl - my_lt, warp);
        eq_base = __shfl_sync(kFull, eq_incl - my_eq, warp);
        below_all = __shfl_sync(kFull, lt_incl, kSelWarps - 1);
    }
    if (threadIdx.x == 0) kdist2[self] = __uint_as_float(kth);

    // ordered emission; a warp stops once its keys below the k-th are out
    // and the tie slots are full
    eq_base += below_all;
    const int lt_end = lt_base + sh.warp_lt[warp];
    for (int64_t j0 = s0; j0 < s1 && (lt_base < lt_end || eq_base < k); j0 += 32) {
        const int64_t j = j0 + lane;
        const bool in = j < s1 && (gram || j != self);
        const unsigned u = in ? row_key(row, cache, cached, j) : 0u;
        const bool is_lt = in && u < kth, is_eq = in && u == kth;
        const unsigned mlt = __ballot_sync(kFull, is_lt), meq = __ballot_sync(kFull, is_eq);
        const unsigned before = (1u << lane) - 1u;
        int slot = -1;
        if (is_lt) slot = lt_base + __popc(mlt & before);
        if (is_eq) slot = eq_base + __popc(meq & before);
        if (slot >= 0 && slot < k) {
            nbr_idx[static_cast<int64_t>(slot) * n + self] = static_cast<int32_t>(j);
            nbr_d2[static_cast<int64_t>(slot) * n + self] = __uint_as_float(u);
        }
        lt_base += __popc(mlt);
        eq_base += __popc(meq);
    }
}

}  // namespace

void distance_tile(const float* xc, int64_t n, int d, int64_t row0, int rows, float* tile,
                   cudaStream_t s) {
    dim3 grid(static_cast<unsigned>(ceil_div(n, kTileBlock)), static_cast<unsigned>(ceil_div(rows, kTileRows)));
    distance_tile_kernel<<<grid, kTileBlock, 0, s>>>(xc, n, d, row0, rows, tile);
    CG_LAUNCH_CHECK();
}

void select_tile_rows(float* tile, const float* norms, int rows, int64_t row_offset, int64_t n, int k, int mode,
                      int32_t* nbr_idx, float* nbr_d2, float* kdist2, cudaStream_t s) {
    if (rows <= 0) return;
    set_max_dynamic_smem(reinterpret_cast<const void*>(row_select_kernel), kRowCache * sizeof(unsigned));
    const int smem = n <= kRowCache ? static_cast<int>(n * sizeof(unsigned)) : 0;
    row_select_kernel<<<rows, kSelThreads, smem, s>>>(tile, norms, rows, row_offset, n, k, mode, nbr_idx, nbr_d2,
                                                      kdist2);
    CG_LAUNCH_CHECK();
}

namespace {
__global__ void iota_rows_kernel(int32_t* __restrict__ rows, int64_t first, int64_t m) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < m;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        rows[i] = static_cast<int32_t>(first + i);
}
}  // namespace

void iota_rows(int32_t* rows, int64_t first, int64_t m, cudaStream_t s) {
    int64_t g = ceil_div(m, 256);
    if (g > 1024) g = 1024;
    iota_rows_kernel<<<static_cast<unsigned>(g), 256, 0, s>>>(rows, first, m);
    CG_LAUNCH_CHECK();
}

// pipeline.cu:33-38: rows = clamp(budget / (4 n), 1, n).
int choose_tile_rows(int64_t n_points, size_t budget_bytes) {
    const size_t row_bytes = static_cast<size_t>(n_points) * sizeof(float);
    size_t rows = budget_bytes / (row_bytes > 0 ? row_bytes : 1);
    if (rows < 1) rows = 1;
    if (rows > static_cast<size_t>(n_points)) rows = static_cast<size_t>(n_points);
    return static_cast<int>(rows);
}

}  // namespace culof_gb300
