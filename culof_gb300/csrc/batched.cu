// Batched LOF over many independent problems in one persistent launch,
// replayed from a CUDA graph.
//
// The reference serves one problem per culof::lof call: a private stream and
// seven cudaMallocs per call (pipeline.cu:148-168), then the pipeline. A loop
// of such calls over thousands of small problems is bound by that per-call
// setup and by launches that cannot fill the GPU. Here one call takes all
// problems (points concatenated, per-problem offsets and k):
//   1. batched centring: the single-problem centring's arithmetic, in the
//      same order (chunks of kCenterChunk rows), for every problem at once;
//   2. a spatial order within each problem (Morton keys over its 8 widest
//      dimensions, two stable radix sorts);
//   3. a persistent k-NN kernel: CTAs pull (problem, 128-row tile) work items
//      from an atomic counter, largest problems first, visit the problem's
//      column tiles nearest first (spiral from the own tile) and select each row's
//      exact k nearest among its problem's points (FP32 direct differences,
//      the oracle's formula, two columns per packed f32x2 instruction) into
//      per-row lists in shared memory;
//   4. batched lrd and scores with the reference's FP64 sums.
// Every problem's scores are bit-identical to a single-problem call. The
// launch sequence of a given batch layout is captured once as a CUDA graph
// and replayed; on first sight of a layout a small autotuner times the k-NN
// kernel's variants (CTAs per SM, one or two column pairs per lane) and
// keeps the fastest.
#include <algorithm>
#include <cstring>
#include <sstream>
#include <vector>

#include "common.cuh"
#include "engine.cuh"
#include "fast.cuh"
#include "sweep_common.cuh"

namespace culof_gb300 {

namespace {

using namespace sweep;

constexpr int kBM = 80;          // list capacity per row: k + 32 free slots (two CTAs per SM)
constexpr int kBMaxK = kBM - 32;
constexpr int kBMaxD = 64;

// ---- batched centring (prep.cu's arithmetic per problem) -------------------

// One thread per (global chunk, feature); chunk g belongs to problem cp[g].
__global__ void bc_partials_kernel(const float* __restrict__ x, const int64_t* __restrict__ off, int d,
                                   const int* __restrict__ cp, const int64_t* __restrict__ coff, int64_t nchunks,
                                   const double* __restrict__ mean, double* __restrict__ partial) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= nchunks * d) return;
    const int64_t g = t / d;
    const int f = static_cast<int>(t % d);
    const int p = cp[g];
    const int64_t c = g - coff[p];
    const int64_t n = off[p + 1] - off[p];
    const float* xp = x + off[p] * d;
    const int64_t begin = c * kCenterChunk;
    const int64_t end = begin + kCenterChunk < n ? begin + kCenterChunk : n;
    double s = 0.0;
    if (mean == nullptr) {
        for (int64_t i = begin; i < end; ++i) s = __dadd_rn(s, static_cast<double>(xp[i * d + f]));
    } else {
        const double m = mean[static_cast<int64_t>(p) * d + f];
        for (int64_t i = begin; i < end; ++i) {
            const double v = __dsub_rn(static_cast<double>(xp[i * d + f]), m);
            s = __dadd_rn(s, __dmul_rn(v, v));
        }
    }
    partial[t] = s;
}

__global__ void bc_finalize_kernel(const double* __restrict__ partial, const int64_t* __restrict__ off,
                                   const int64_t* __restrict__ coff, int num, int d, int mode,
                                   double* __restrict__ mean, double* __restrict__ inv_std) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= static_cast<int64_t>(num) * d) return;
    const int p = static_cast<int>(t / d);
    const int f = static_cast<int>(t % d);
    double total = 0.0;
    for (int64_t c = coff[p]; c < coff[p + 1]; ++c) total = __dadd_rn(total, partial[c * d + f]);
    const double dn = static_cast<double>(off[p + 1] - off[p]);
    if (mode == 0) {
        mean[t] = __ddiv_rn(total, dn);
        inv_std[t] = 1.0;
    } else {
        const double sd = __dsqrt_rn(__ddiv_rn(total, dn));
        inv_std[t] = (sd > 1e-12) ? __ddiv_rn(1.0, sd) : 1.0;
    }
}

__global__ void bc_apply_kernel(const float* __restrict__ x, int64_t ntot, int d, const int* __restrict__ pid,
                                const double* __restrict__ mean, const double* __restrict__ inv_std,
                                float* __restrict__ xc) {
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < ntot * d;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t i = t / d;
        const int f = static_cast<int>(t % d);
        const int64_t pf = static_cast<int64_t>(pid[i]) * d + f;
        xc[t] = __double2float_rn(__dmul_rn(__dsub_rn(static_cast<double>(x[t]), mean[pf]), inv_std[pf]));
    }
}

// ---- spatial order within each problem -----------------------------------------

__device__ __forceinline__ unsigned flip_f(float f) {
    const unsigned u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unflip_f(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

constexpr int kMortonDimsB = 8;

// One block per problem: per-dimension range of its centred points, then
// the (up to) 8 widest dimensions, widest first (ties by index).
__global__ void bm_minmax_kernel(const float* __restrict__ xc, const int64_t* __restrict__ off, int d,
                                 float* __restrict__ pmm, int* __restrict__ pdims) {
    __shared__ unsigned lo[kBMaxD], hi[kBMaxD];
    const int p = blockIdx.x;
    for (int f = threadIdx.x; f < d; f += blockDim.x) {
        lo[f] = 0xFFFFFFFFu;
        hi[f] = 0u;
    }
    __syncthreads();
    const int64_t b = off[p], e = off[p + 1];
    for (int64_t t = threadIdx.x; t < (e - b) * d; t += blockDim.x) {
        const int f = static_cast<int>(t % d);
        const unsigned k = flip_f(xc[b * d + t]);
        atomicMin(&lo[f], k);
        atomicMax(&hi[f], k);
    }
    __syncthreads();
    for (int f = threadIdx.x; f < d; f += blockDim.x) {
        pmm[(static_cast<int64_t>(p) * d + f) * 2] = unflip_f(lo[f]);
        pmm[(static_cast<int64_t>(p) * d + f) * 2 + 1] = unflip_f(hi[f]);
    }
    if (threadIdx.x == 0) {
        const int m = d < kMortonDimsB ? d : kMortonDimsB;
        int chosen[kMortonDimsB];
        for (int j = 0; j < m; ++j) {
            int best = -1;
            float span = -1.0f;
            for (int f = 0; f < d; ++f) {
                bool taken = false;
                for (int q = 0; q < j; ++q) taken |= chosen[q] == f;
                const float sp = unflip_f(hi[f]) - unflip_f(lo[f]);
                if (!taken && sp > span) {
                    span = sp;
                    best = f;
                }
            }
            chosen[j] = best;
            pdims[p * kMortonDimsB + j] = best;
        }
    }
}

// Morton key of each point over its problem's chosen dimensions.
__global__ void bm_morton_kernel(const float* __restrict__ xc, int64_t ntot, int d, const int* __restrict__ pid,
                                 const float* __restrict__ pmm, const int* __restrict__ pdims,
                                 unsigned* __restrict__ keys, unsigned* __restrict__ vals) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < ntot;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int p = pid[i];
        const int m = d < kMortonDimsB ? d : kMortonDimsB;
        const int bits = (32 / m) < 10 ? 32 / m : 10;
        unsigned q[kMortonDimsB];
        for (int j = 0; j < m; ++j) {
            const int f = pdims[p * kMortonDimsB + j];
            const float lo = pmm[(static_cast<int64_t>(p) * d + f) * 2], hi = pmm[(static_cast<int64_t>(p) * d + f) * 2 + 1];
            const float span = hi - lo;
            float t = span > 0.0f ? (xc[i * d + f] - lo) / span : 0.0f;
            t = fminf(fmaxf(t, 0.0f), 1.0f);
            q[j] = static_cast<unsigned>(t * static_cast<float>((1u << bits) - 1u) + 0.5f);
        }
        unsigned key = 0u;
        for (int bt = bits - 1; bt >= 0; --bt)
            for (int j = 0; j < m; ++j) key = (key << 1) | ((q[j] >> bt) & 1u);
        keys[i] = key;
        vals[i] = static_cast<unsigned>(i);
    }
}

__global__ void bm_pidkey_kernel(int64_t ntot, const int* __restrict__ pid, const unsigned* __restrict__ vals,
                                 unsigned* __restrict__ keys) {
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < ntot;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        keys[i] = static_cast<unsigned>(pid[vals[i]]);
}

// Sorted coordinates and, per sorted position, the point's original index
// within its problem.
__global__ void bm_gather_kernel(const float* __restrict__ xc, int64_t ntot, int d, const unsigned* __restrict__ perm,
                                 const int* __restrict__ pid, const int64_t* __restrict__ off, float* __restrict__ xs,
                                 unsigned* __restrict__ lidx) {
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < ntot * d;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t i = t / d;
        const int f = static_cast<int>(t % d);
        const unsigned src = perm[i];
        xs[t] = xc[static_cast<int64_t>(src) * d + f];
        if (f == 0) lidx[i] = static_cast<unsigned>(src - off[pid[src]]);
    }
}

// One warp per (problem, tile of 128 sorted points): the tile's bounding box,
// tbox[tile_off[p] + t][2][d] (lo, hi).
__global__ void bm_tilebox_kernel(const float* __restrict__ xs, const int64_t* __restrict__ off, int d,
                                  const int* __restrict__ tpid, const int64_t* __restrict__ toff, int64_t ntiles,
                                  float* __restrict__ tbox) {
    const int lane = threadIdx.x & 31;
    const int64_t g = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (g >= ntiles) return;
    const int p = tpid[g];
    const int64_t t = g - toff[p];
    const int64_t b = off[p] + t * kCT;
    const int64_t e = (b + kCT < off[p + 1]) ? b + kCT : off[p + 1];
    for (int f = 0; f < d; ++f) {
        float lo = __int_as_float(0x7f800000), hi = __int_as_float(0xff800000);
        for (int64_t i = b + lane; i < e; i += 32) {
            const float v = xs[i * d + f];
            lo = fminf(lo, v);
            hi = fmaxf(hi, v);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        if (lane == 0) {
            tbox[(g * 2) * d + f] = lo;
            tbox[(g * 2 + 1) * d + f] = hi;
        }
    }
}

// Pruning margin for d <= 64: the float32 direct-difference distance of two
// points at real squared distance T >= LB is >= T (1 - (d + 2) 2^-24) >
// LB (1 - 2^-17), so a tile whose rounded-down box gap times (1 - 2^-17)
// exceeds every row's k-th distance holds no candidate.
constexpr float kBPruneShrink = 0.9999923706054688f;  // 1 - 2^-17

// Rounded-down squared gap between box a (lo, hi) and box b, lanes over
// dimensions, round-down sums; the result is warp-uniform.
__device__ __forceinline__ float gap2_rd(const float* a_lo, const float* a_hi, const float* b_lo, const float* b_hi,
                                         int d) {
    const int lane = threadIdx.x & 31;
    float g = 0.0f;
    for (int f = lane; f < d; f += 32) {
        const float gap = fmaxf(0.0f, fmaxf(__fsub_rd(b_lo[f], a_hi[f]), __fsub_rd(a_lo[f], b_hi[f])));
        g = __fadd_rd(g, __fmul_rd(gap, gap));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) g = __fadd_rd(g, __shfl_xor_sync(0xffffffffu, g, o));
    return g;
}

// ---- persistent k-NN ---------------------------------------------------------

template <int DP>
struct BatchSmem {
    RowLists<kBM> L;
    uint64_t rows2[kRT][DP];         // this item's rows, each coordinate duplicated into both halves
    uint64_t cols2[kCT / 2][DP + 1];  // one column tile as packed column pairs (odd stride)
    float wbox[kWarps][2][DP];        // each warp's row box
    float cbox[2][DP];                // the item's row box
    float tb[2][2][DP];               // column tile box, by tile parity (warp 0 runs at most one tile ahead)
    int skip_tile[2];
    int item;
};

// Append this lane's key for row r (if it beats the row's k-th key), keeping
// 32 free slots: warp-uniform.
__device__ __forceinline__ void offer(RowLists<kBM>& L, int r, uint64_t key, int k) {
    const int lane = threadIdx.x & 31;
    bool pass = key < L.kth[r];
    unsigned m = __ballot_sync(0xffffffffu, pass);
    if (!m) return;
    if (L.cnt[r] > kBM - 32) {
        compact_row<kBM>(L, r, k, 0.0f, 8);
        pass = key < L.kth[r];
        m = __ballot_sync(0xffffffffu, pass);
        if (!m) return;
    }
    const int c = L.cnt[r];
    if (pass) L.list[r][c + __popc(m & ((1u << lane) - 1u))] = key;
    __syncwarp();
    if (lane == 0) L.cnt[r] = c + __popc(m);
    __syncwarp();
}

// Offer a row's 2 * CP keys (one warp-uniform test first).
template <int CP>
__device__ __forceinline__ void offer_row(RowLists<kBM>& L, int r, const uint64_t (&key)[2 * CP], int k) {
    uint64_t mn = key[0];
#pragma unroll
    for (int q = 1; q < 2 * CP; ++q) mn = key[q] < mn ? key[q] : mn;
    if (!__any_sync(0xffffffffu, mn < L.kth[r])) return;
#pragma unroll
    for (int q = 0; q < 2 * CP; ++q) offer(L, r, key[q], k);
}

// Each warp owns 16 rows of the item. The CTA stages the problem's columns
// in tiles of 128 (packed column pairs in shared memory); per pass a lane
// holds CP column pairs in registers (packed f32x2 per dimension), so two
// rows x CP pairs give 2 * CP independent packed FMA chains. Distances are
// the oracle's direct-difference chain, exactly (per-lane IEEE sub.rn /
// fma.rn).
// Two CTAs per SM (what the shared memory allows up to DP = 32); without the
// minimum, the compiler gives the DP = 8 forms 64 registers and spills.
template <int DP, int CP>
__global__ void __launch_bounds__(kThreads, DP <= 32 ? 2 : 1)
batched_knn_kernel(const float* __restrict__ xc, const unsigned* __restrict__ lidx, const int64_t* __restrict__ off,
                   const int* __restrict__ ks, const int64_t* __restrict__ nkoff, const uint2* __restrict__ items,
                   int nitems, int d, unsigned* __restrict__ counter, int32_t* __restrict__ nbr_idx,
                   float* __restrict__ nbr_d2, float* __restrict__ kdist2, const float* __restrict__ tbox,
                   const int64_t* __restrict__ toff) {
    extern __shared__ __align__(16) unsigned char braw[];
    BatchSmem<DP>& sh = *reinterpret_cast<BatchSmem<DP>*>(braw);
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    constexpr int kTile = 64 * CP;
    for (;;) {
        if (tid == 0) sh.item = static_cast<int>(atomicAdd(counter, 1u));
        __syncthreads();
        const int item = sh.item;
        if (item >= nitems) break;
        const int p = static_cast<int>(items[item].x);
        const int T = static_cast<int>(items[item].y);
        const int64_t base = off[p];
        const int n = static_cast<int>(off[p + 1] - base);
        const int k = ks[p];
        const float* xp = xc + base * d;
        const int r0 = T * kRT;
        for (int i = tid; i < kRT * DP; i += kThreads) {
            const int r = i / DP, f = i % DP;
            sh.rows2[r][f] = dup2((r0 + r < n && f < d) ? xp[static_cast<int64_t>(r0 + r) * d + f] : 0.0f);
        }
        if (tid < kRT) {
            sh.L.cnt[tid] = 0;
            sh.L.sorted[tid] = 0;
            sh.L.kth[tid] = kKeyMax;
            sh.L.row_norm[tid] = 0.0f;
        }
        __syncthreads();
        const int rw = warp * kRowsPerWarp;
        // row boxes: this warp's 16 rows and (warp 0, after the barrier) the item's
        {
            const int r = rw + (lane & 15);
            const bool rv = r0 + r < n;
            for (int f = 0; f < d; ++f) {
                const float v = lo_f(sh.rows2[r][f]);
                float lo = rv ? v : __int_as_float(0x7f800000), hi = rv ? v : __int_as_float(0xff800000);
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
        }
        __syncthreads();
        if (tid < d) {
            float lo = __int_as_float(0x7f800000), hi = __int_as_float(0xff800000);
            for (int w = 0; w < kWarps; ++w) {
                lo = fminf(lo, sh.wbox[w][0][tid]);
                hi = fmaxf(hi, sh.wbox[w][1][tid]);
            }
            sh.cbox[0][tid] = lo;
            sh.cbox[1][tid] = hi;
        }
        const unsigned* li = lidx + base;  // original index of each sorted position
        const int ntp = (n + kCT - 1) / kCT;
        // column tiles in spiral order from the item's own tile: near points
        // first, so the lists fill with good neighbours early
#pragma unroll 1
        for (int qt = 0; qt < ntp; ++qt) {
            const int ct = spiral_tile(T, qt, ntp);
            const int c0 = ct * kCT;
            // prune (warp 0): the tile is farther than every row's k-th distance
            // (bounding boxes only pay in low dimensions: DP <= 8)
            const int par = qt & 1;
            if (DP <= 8 && warp == 0) {
                const float* g = tbox + (toff[p] + ct) * 2 * d;
                for (int f = lane; f < d; f += 32) {
                    sh.tb[par][0][f] = g[f];
                    sh.tb[par][1][f] = g[d + f];
                }
                float km = __int_as_float(0xff800000);
                for (int r = lane; r < kRT; r += 32) {
                    if (r0 + r < n) {
                        const uint64_t kk = sh.L.kth[r];
                        km = fmaxf(km, kk == kKeyMax ? __int_as_float(0x7f800000) : __uint_as_float(key_bits(kk)));
                    }
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) km = fmaxf(km, __shfl_xor_sync(0xffffffffu, km, o));
                __syncwarp();
                const float g2 = gap2_rd(sh.cbox[0], sh.cbox[1], sh.tb[par][0], sh.tb[par][1], d);
                if (lane == 0) sh.skip_tile[par] = __fmul_rd(g2, kBPruneShrink) > km ? 1 : 0;
            }
            if (DP <= 8) {
                __syncthreads();
                if (sh.skip_tile[par]) continue;
            }
            // this warp's rows may all be beyond the tile
            bool wskip = false;
            if (DP <= 8) {
                float wk = __int_as_float(0xff800000);
                if (lane < kRowsPerWarp && r0 + rw + lane < n) {
                    const uint64_t kk = sh.L.kth[rw + lane];
                    wk = kk == kKeyMax ? __int_as_float(0x7f800000) : __uint_as_float(key_bits(kk));
                }
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) wk = fmaxf(wk, __shfl_xor_sync(0xffffffffu, wk, o));
                wskip = __fmul_rd(gap2_rd(sh.wbox[warp][0], sh.wbox[warp][1], sh.tb[par][0], sh.tb[par][1], d),
                                  kBPruneShrink) > wk;
            }
            // the CTA stages 128 columns (coalesced) as packed pairs
            for (int i = tid; i < kCT * DP; i += kThreads) {
                const int c = i / DP, f = i % DP;
                const float v = (c0 + c < n && f < d) ? xp[static_cast<int64_t>(c0 + c) * d + f] : 0.0f;
                reinterpret_cast<float*>(&sh.cols2[c >> 1][f])[c & 1] = v;
            }
            __syncthreads();
#pragma unroll 1
            for (int sub = 0; sub < (wskip ? 0 : kCT); sub += kTile) {
            uint64_t cp[CP][DP];
            int cc[CP];
            // per column: its original index in the key's low half, or all
            // ones (a key of kKeyMax) for columns beyond the problem
            uint64_t cidx[2 * CP];
#pragma unroll
            for (int q = 0; q < CP; ++q) {
                const int pr = (sub >> 1) + 32 * q + lane;  // column pair index in the tile
                cc[q] = c0 + 2 * pr;
#pragma unroll
                for (int f = 0; f < DP; ++f) cp[q][f] = sh.cols2[pr][f];
                cidx[2 * q] = cc[q] < n ? static_cast<uint64_t>(li[cc[q]]) : kKeyMax;
                cidx[2 * q + 1] = cc[q] + 1 < n ? static_cast<uint64_t>(li[cc[q] + 1]) : kKeyMax;
            }
            const bool own = c0 == r0;  // the only tile holding the rows' own points
#pragma unroll 1
            for (int rr = 0; rr < kRowsPerWarp; rr += 2) {
                const int r = rw + rr;
                if (r0 + r >= n) break;  // warp-uniform: rows beyond the problem
                uint64_t s[2][CP];
#pragma unroll
                for (int h = 0; h < 2; ++h)
#pragma unroll
                    for (int q = 0; q < CP; ++q) s[h][q] = 0;
                // dimensions past d are zero in both operands: each adds
                // fma(0, 0, s) = s, so the chain over all DP equals the
                // oracle's chain over d
#pragma unroll
                for (int f = 0; f < DP; ++f) {
                    const uint64_t a0 = sh.rows2[r][f], a1 = sh.rows2[r + 1][f];
#pragma unroll
                    for (int q = 0; q < CP; ++q) {
                        uint64_t t0, t1;
                        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(t0) : "l"(a0), "l"(cp[q][f]));
                        asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(t1) : "l"(a1), "l"(cp[q][f]));
                        s[0][q] = fma2(t0, t0, s[0][q]);
                        s[1][q] = fma2(t1, t1, s[1][q]);
                    }
                }
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const int gr = r0 + r + h;
                    if (gr >= n) break;  // warp-uniform
                    // a key can beat the row's k-th key only if its distance
                    // is at most the k-th distance: test the distances first
                    const uint64_t kk = sh.L.kth[r + h];
                    const float kd = kk == kKeyMax ? __int_as_float(0x7f800000) : __uint_as_float(key_bits(kk));
                    bool maybe = false;
#pragma unroll
                    for (int q = 0; q < CP; ++q) maybe |= (lo_f(s[h][q]) <= kd) | (hi_f(s[h][q]) <= kd);
                    if (!__any_sync(0xffffffffu, maybe)) continue;
                    uint64_t key[2 * CP];
#pragma unroll
                    for (int q = 0; q < CP; ++q) {
                        key[2 * q] = (static_cast<uint64_t>(__float_as_uint(lo_f(s[h][q]))) << 32) | cidx[2 * q];
                        key[2 * q + 1] = (static_cast<uint64_t>(__float_as_uint(hi_f(s[h][q]))) << 32) | cidx[2 * q + 1];
                        if (own) {  // a row is not its own neighbour
                            if (cc[q] == gr) key[2 * q] = kKeyMax;
                            if (cc[q] + 1 == gr) key[2 * q + 1] = kKeyMax;
                        }
                    }
                    offer_row<CP>(sh.L, r + h, key, k);
                }
            }
            }
            __syncthreads();
        }
        // the k best per row, written in the reference's slot order
        for (int rr = 0; rr < kRowsPerWarp; ++rr) {
            const int r = rw + rr;
            if (r0 + r >= n) break;
            const int il = static_cast<int>(li[r0 + r]);  // the row's original index
            compact_row<kBM>(sh.L, r, k, 0.0f, 8);
            const uint64_t kth = sh.L.list[r][k - 1];
            const uint32_t kbits = key_bits(kth);
            int below = 0;
            for (int e = lane; e < k; e += 32) below += key_bits(sh.L.list[r][e]) < kbits ? 1 : 0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) below += __shfl_xor_sync(0xffffffffu, below, o);
            int32_t* oi = nbr_idx + nkoff[p];
            float* od = nbr_d2 + nkoff[p];
            for (int e = lane; e < k; e += 32) {
                const uint64_t y = sh.L.list[r][e];
                int slot = e;
                if (e < below) {
                    const uint32_t yi = key_index(y);
                    slot = 0;
                    for (int q = 0; q < below; ++q) slot += key_index(sh.L.list[r][q]) < yi ? 1 : 0;
                }
                oi[static_cast<int64_t>(slot) * n + il] = static_cast<int32_t>(key_index(y));
                od[static_cast<int64_t>(slot) * n + il] = __uint_as_float(key_bits(y));
            }
            if (lane == 0) kdist2[base + il] = __uint_as_float(kbits);
        }
        __syncthreads();
    }
}

// ---- batched lrd and scores (lof.cu's arithmetic, local indices) -------------

__global__ void bl_lrd_kernel(int64_t ntot, const int* __restrict__ pid, const int64_t* __restrict__ off,
                              const int* __restrict__ ks, const int64_t* __restrict__ nkoff,
                              const int32_t* __restrict__ nbr_idx, const float* __restrict__ nbr_d2,
                              const float* __restrict__ kdist2, float* __restrict__ lrd) {
    const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= ntot) return;
    const int p = pid[g];
    const int64_t base = off[p];
    const int64_t n = off[p + 1] - base, i = g - base;
    const int k = ks[p];
    const int32_t* ni = nbr_idx + nkoff[p];
    const float* nd = nbr_d2 + nkoff[p];
    double sum = 0.0;
    for (int t = 0; t < k; ++t) {
        const int64_t o = static_cast<int64_t>(t) * n + i;
        const int32_t j = ni[o];
        const float kj = (j >= 0 && j < n) ? kdist2[base + j] : __int_as_float(0x7fc00000);
        sum = __dadd_rn(sum, __dsqrt_rn(static_cast<double>(fmaxf(kj, nd[o]))));
    }
    lrd[g] = __double2float_rn(__ddiv_rn(1.0, __dadd_rn(__ddiv_rn(sum, static_cast<double>(k)), 1e-10)));
}

__global__ void bl_score_kernel(int64_t ntot, const int* __restrict__ pid, const int64_t* __restrict__ off,
                                const int* __restrict__ ks, const int64_t* __restrict__ nkoff,
                                const int32_t* __restrict__ nbr_idx, const float* __restrict__ lrd,
                                float* __restrict__ scores) {
    const int64_t g = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (g >= ntot) return;
    const int p = pid[g];
    const int64_t base = off[p];
    const int64_t n = off[p + 1] - base, i = g - base;
    const int k = ks[p];
    const int32_t* ni = nbr_idx + nkoff[p];
    const double self = static_cast<double>(lrd[g]);
    double sum = 0.0;
    for (int t = 0; t < k; ++t) {
        const int32_t j = ni[static_cast<int64_t>(t) * n + i];
        const double lj = (j >= 0 && j < n) ? static_cast<double>(lrd[base + j]) : __longlong_as_double(0x7ff8000000000000ll);
        sum = __dadd_rn(sum, __ddiv_rn(lj, self));
    }
    scores[g] = __double2float_rn(__ddiv_rn(sum, static_cast<double>(k)));
}

__global__ void pid_kernel(const int64_t* __restrict__ off, int num, int* __restrict__ pid) {
    // one block per problem
    for (int p = blockIdx.x; p < num; p += gridDim.x)
        for (int64_t i = off[p] + threadIdx.x; i < off[p + 1]; i += blockDim.x) pid[i] = p;
}

int dp_for(int d) { return d <= 4 ? 4 : d <= 8 ? 8 : d <= 16 ? 16 : d <= 32 ? 32 : 64; }

template <int DP, int CP>
void launch_knn_t(int grid, const BatchDev& b, cudaStream_t s) {
    const size_t smem = sizeof(BatchSmem<DP>);
    set_max_dynamic_smem(reinterpret_cast<const void*>(batched_knn_kernel<DP, CP>), static_cast<int>(smem));
    batched_knn_kernel<DP, CP><<<grid, kThreads, smem, s>>>(b.xs, b.lidx, b.off, b.ks, b.nkoff, b.items, b.nitems,
                                                           b.d, b.counter, b.nbr, b.d2, b.kd, b.tbox, b.toff);
    CG_LAUNCH_CHECK();
}

// cp2: two column pairs per lane (d <= 16), else one.
void launch_knn(int dp, bool cp2, int grid, const BatchDev& b, cudaStream_t s) {
    switch (dp) {
        case 4: cp2 ? launch_knn_t<4, 2>(grid, b, s) : launch_knn_t<4, 1>(grid, b, s); break;
        case 8: cp2 ? launch_knn_t<8, 2>(grid, b, s) : launch_knn_t<8, 1>(grid, b, s); break;
        case 16: cp2 ? launch_knn_t<16, 2>(grid, b, s) : launch_knn_t<16, 1>(grid, b, s); break;
        case 32: launch_knn_t<32, 1>(grid, b, s); break;
        case 64: launch_knn_t<64, 1>(grid, b, s); break;
        default: throw Error(kInternal, "bad padded dimension");
    }
}

template <int DP>
size_t knn_smem() { return sizeof(BatchSmem<DP>); }
size_t knn_smem_for(int dp) {
    switch (dp) {
        case 4: return knn_smem<4>();
        case 8: return knn_smem<8>();
        case 16: return knn_smem<16>();
        case 32: return knn_smem<32>();
        default: return knn_smem<64>();
    }
}

int grid_cap(int64_t items) {
    int64_t g = ceil_div(items, 256);
    if (g > 152 * 16) g = 152 * 16;
    return static_cast<int>(g < 1 ? 1 : g);
}

}  // namespace

// ---- host orchestration --------------------------------------------------------

void Engine::batch_plan(int num, const int64_t* offsets, const int* ks, int d, bool normalize) {
    if (num < 1) throw Error(kInvalidArgument, "num_problems must be >= 1");
    if (!offsets || !ks) throw Error(kInvalidArgument, "offsets and ks must not be null");
    if (d < 1 || d > kBMaxD) throw Error(kInvalidArgument, "the batched path takes 1 <= n_dims <= 64");
    if (offsets[0] != 0) throw Error(kInvalidArgument, "offsets[0] must be 0");
    BatchPlan& P = bplan_;
    P.num = num;
    P.d = d;
    P.normalize = normalize;
    P.off.assign(offsets, offsets + num + 1);
    P.ks.assign(ks, ks + num);
    P.nkoff.assign(num + 1, 0);
    P.coff.assign(num + 1, 0);
    P.toff.assign(num + 1, 0);
    std::vector<int> tp;
    std::vector<std::pair<int64_t, uint2>> items;
    std::vector<int> cp;
    for (int p = 0; p < num; ++p) {
        const int64_t n = offsets[p + 1] - offsets[p];
        const int k = ks[p];
        if (n < 2 || n > 0x7FFFFFFFll) {
            std::ostringstream os;
            os << "problem " << p << ": n_points must be >= 2 (got " << n << ")";
            throw Error(kInvalidArgument, os.str());
        }
        if (k < 1 || k >= n || k > kBMaxK) {
            std::ostringstream os;
            os << "problem " << p << ": k must satisfy 1 <= k <= n_points - 1 and k <= " << kBMaxK << " (got k=" << k
               << ", n_points=" << n << ")";
            throw Error(kInvalidArgument, os.str());
        }
        P.nkoff[p + 1] = P.nkoff[p] + n * k;
        const int64_t chunks = ceil_div(n, kCenterChunk);
        P.coff[p + 1] = P.coff[p] + chunks;
        for (int64_t c = 0; c < chunks; ++c) cp.push_back(p);
        const int64_t tiles = ceil_div(n, kRT);
        P.toff[p + 1] = P.toff[p] + tiles;
        for (int64_t t = 0; t < tiles; ++t) {
            items.push_back({n, make_uint2(static_cast<unsigned>(p), static_cast<unsigned>(t))});
            tp.push_back(p);
        }
    }
    // largest problems first: their items are the longest, the tail stays short
    std::stable_sort(items.begin(), items.end(),
                     [](const std::pair<int64_t, uint2>& a, const std::pair<int64_t, uint2>& b) { return a.first > b.first; });
    P.items.resize(items.size());
    for (size_t i = 0; i < items.size(); ++i) P.items[i] = items[i].second;
    P.ntot = offsets[num];
    P.nchunks = P.coff[num];
    // device copies of the plan (synchronous, before any capture)
    cudaStream_t s = stream_;
    BatchDev& b = bdev_;
    b.off = bplan_off_.as<int64_t>(num + 1);
    b.nkoff = bplan_nkoff_.as<int64_t>(num + 1);
    b.coff = bplan_coff_.as<int64_t>(num + 1);
    b.ks = bplan_ks_.as<int>(num);
    b.items = bplan_items_.as<uint2>(P.items.size());
    b.cp = bplan_cp_.as<int>(cp.size() ? cp.size() : 1);
    b.toff = bplan_toff_.as<int64_t>(num + 1);
    b.tpid = bplan_tpid_.as<int>(tp.size());
    b.ntiles = static_cast<int64_t>(tp.size());
    CG_CUDA(cudaMemcpyAsync(b.toff, P.toff.data(), sizeof(int64_t) * (num + 1), cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(b.tpid, tp.data(), sizeof(int) * tp.size(), cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(b.off, P.off.data(), sizeof(int64_t) * (num + 1), cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(b.nkoff, P.nkoff.data(), sizeof(int64_t) * (num + 1), cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(b.coff, P.coff.data(), sizeof(int64_t) * (num + 1), cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(b.ks, P.ks.data(), sizeof(int) * num, cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(b.items, P.items.data(), sizeof(uint2) * P.items.size(), cudaMemcpyHostToDevice, s));
    CG_CUDA(cudaMemcpyAsync(b.cp, cp.data(), sizeof(int) * cp.size(), cudaMemcpyHostToDevice, s));
    b.nitems = static_cast<int>(P.items.size());
    b.d = d;
    // workspaces
    b.pid = bpid_.as<int>(P.ntot);
    b.xc = bxc_.as<float>(static_cast<size_t>(P.ntot) * d);
    b.partial = bpartial_.as<double>(static_cast<size_t>(P.nchunks) * d);
    b.mean = bmean_.as<double>(static_cast<size_t>(num) * d);
    b.inv = binv_.as<double>(static_cast<size_t>(num) * d);
    b.nbr = bnbr_.as<int32_t>(P.nkoff[num]);
    b.d2 = bd2_.as<float>(P.nkoff[num]);
    b.kd = bkd_.as<float>(P.ntot);
    b.lrd = blrd_.as<float>(P.ntot);
    b.counter = bcounter_.as<unsigned>(1);
    b.xs = bxs_.as<float>(static_cast<size_t>(P.ntot) * d);
    b.lidx = blidx_.as<unsigned>(P.ntot);
    b.pmm = bpmm_.as<float>(static_cast<size_t>(num) * d * 2);
    b.pdims = bpdims_.as<int>(static_cast<size_t>(num) * kMortonDimsB);
    b.skeys = bskeys_.as<unsigned>(2 * static_cast<size_t>(P.ntot));
    b.svals = bsvals_.as<unsigned>(2 * static_cast<size_t>(P.ntot));
    b.scounts = bscounts_.as<unsigned>(sort_pairs_counts(P.ntot));
    b.tbox = btbox_.as<float>(static_cast<size_t>(b.ntiles) * 2 * d);
    pid_kernel<<<num < 4096 ? num : 4096, 256, 0, s>>>(b.off, num, b.pid);
    CG_LAUNCH_CHECK();
    CG_CUDA(cudaStreamSynchronize(s));
    bgraph_valid_ = false;
    btuned_ = false;
}

void Engine::batch_launch(const float* d_x, float* d_scores) {
    const BatchPlan& P = bplan_;
    BatchDev& b = bdev_;
    cudaStream_t s = stream_;
    const int d = P.d;
    const int64_t cd = P.nchunks * d;
    bc_partials_kernel<<<static_cast<unsigned>(ceil_div(cd, 256)), 256, 0, s>>>(d_x, b.off, d, b.cp, b.coff,
                                                                                 P.nchunks, nullptr, b.partial);
    CG_LAUNCH_CHECK();
    bc_finalize_kernel<<<static_cast<unsigned>(ceil_div(static_cast<int64_t>(P.num) * d, 128)), 128, 0, s>>>(
        b.partial, b.off, b.coff, P.num, d, 0, b.mean, b.inv);
    CG_LAUNCH_CHECK();
    if (P.normalize) {
        bc_partials_kernel<<<static_cast<unsigned>(ceil_div(cd, 256)), 256, 0, s>>>(d_x, b.off, d, b.cp, b.coff,
                                                                                     P.nchunks, b.mean, b.partial);
        CG_LAUNCH_CHECK();
        bc_finalize_kernel<<<static_cast<unsigned>(ceil_div(static_cast<int64_t>(P.num) * d, 128)), 128, 0, s>>>(
            b.partial, b.off, b.coff, P.num, d, 1, b.mean, b.inv);
        CG_LAUNCH_CHECK();
    }
    bc_apply_kernel<<<grid_cap(P.ntot * d), 256, 0, s>>>(d_x, P.ntot, d, b.pid, b.mean, b.inv, b.xc);
    CG_LAUNCH_CHECK();
    // spatial order within each problem: Morton keys, stable sort by key,
    // then stable sort by problem (keeps each problem's range in place)
    bm_minmax_kernel<<<P.num, 256, 0, s>>>(b.xc, b.off, d, b.pmm, b.pdims);
    CG_LAUNCH_CHECK();
    bm_morton_kernel<<<grid_cap(P.ntot), 256, 0, s>>>(b.xc, P.ntot, d, b.pid, b.pmm, b.pdims, b.skeys, b.svals);
    CG_LAUNCH_CHECK();
    unsigned* vs = nullptr;
    unsigned* ks1 = sort_pairs_stable(b.skeys, b.svals, b.skeys + P.ntot, b.svals + P.ntot, P.ntot, 32, b.scounts, s, &vs);
    unsigned* kother = ks1 == b.skeys ? b.skeys + P.ntot : b.skeys;
    unsigned* vother = vs == b.svals ? b.svals + P.ntot : b.svals;
    bm_pidkey_kernel<<<grid_cap(P.ntot), 256, 0, s>>>(P.ntot, b.pid, vs, ks1);
    CG_LAUNCH_CHECK();
    int pbits = 8;
    while (pbits < 32 && (static_cast<int64_t>(1) << pbits) < P.num) pbits += 8;
    unsigned* perm = nullptr;
    sort_pairs_stable(ks1, vs, kother, vother, P.ntot, pbits, b.scounts, s, &perm);
    bm_gather_kernel<<<grid_cap(P.ntot * d), 256, 0, s>>>(b.xc, P.ntot, d, perm, b.pid, b.off, b.xs, b.lidx);
    CG_LAUNCH_CHECK();
    bm_tilebox_kernel<<<static_cast<unsigned>(ceil_div(b.ntiles, 8)), 256, 0, s>>>(b.xs, b.off, d, b.tpid, b.toff,
                                                                                   b.ntiles, b.tbox);
    CG_LAUNCH_CHECK();
    CG_CUDA(cudaMemsetAsync(b.counter, 0, sizeof(unsigned), s));
    launch_knn(dp_for(d), btune_packed_, btune_grid_, b, s);
    bl_lrd_kernel<<<static_cast<unsigned>(ceil_div(P.ntot, 256)), 256, 0, s>>>(P.ntot, b.pid, b.off, b.ks, b.nkoff,
                                                                               b.nbr, b.d2, b.kd, b.lrd);
    CG_LAUNCH_CHECK();
    bl_score_kernel<<<static_cast<unsigned>(ceil_div(P.ntot, 256)), 256, 0, s>>>(P.ntot, b.pid, b.off, b.ks,
                                                                                 b.nkoff, b.nbr, b.lrd, d_scores);
    CG_LAUNCH_CHECK();
}

// Time the k-NN kernel's variants on this batch (once per layout).
void Engine::batch_autotune(const float* d_x, float* d_scores) {
    int sms = 152;
    CG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    const int dp = dp_for(bplan_.d);
    const size_t smem = knn_smem_for(dp);
    int max_per_sm = static_cast<int>(227 * 1024 / (smem + 1024));
    if (max_per_sm < 1) max_per_sm = 1;
    if (max_per_sm > 2) max_per_sm = 2;
    cudaEvent_t e0, e1;
    CG_CUDA(cudaEventCreate(&e0));
    CG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (float& t : btune_ms_) t = -1.0f;
    for (int per = 1; per <= max_per_sm; ++per) {
        for (int packed = 0; packed <= (dp <= 16 ? 1 : 0); ++packed) {
            btune_grid_ = per * sms;
            btune_packed_ = packed != 0;
            batch_launch(d_x, d_scores);  // warm (first use configures the kernel)
            CG_CUDA(cudaEventRecord(e0, stream_));
            batch_launch(d_x, d_scores);
            CG_CUDA(cudaEventRecord(e1, stream_));
            CG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            CG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            btune_ms_[2 * (per - 1) + packed] = ms;
            if (ms < best) {
                best = ms;
                bbest_grid_ = btune_grid_;
                bbest_packed_ = btune_packed_;
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    btune_grid_ = bbest_grid_;
    btune_packed_ = bbest_packed_;
    btuned_ = true;
}

bool Engine::batch_same_plan(int num, const int64_t* offsets, const int* ks, int d, bool normalize) const {
    const BatchPlan& P = bplan_;
    if (P.num != num || P.d != d || P.normalize != normalize) return false;
    if (std::memcmp(P.off.data(), offsets, sizeof(int64_t) * (num + 1)) != 0) return false;
    return std::memcmp(P.ks.data(), ks, sizeof(int) * num) == 0;
}

void Engine::lof_batched_device(int num, const int64_t* offsets, const int* ks, const float* d_x, int d,
                                bool normalize, float* d_scores) {
    if (!d_x || !d_scores) throw Error(kInvalidArgument, "device pointers must not be null");
    CG_CUDA(cudaSetDevice(device_));
    if (!(bplan_.num > 0 && batch_same_plan(num, offsets, ks, d, normalize))) batch_plan(num, offsets, ks, d, normalize);
    if (!btuned_) batch_autotune(d_x, d_scores);
    if (!use_graphs_) {
        batch_launch(d_x, d_scores);
        return;
    }
    if (!bgraph_valid_ || bgraph_x_ != d_x || bgraph_scores_ != d_scores || bgraph_stream_ != stream_) {
        if (bgraph_exec_) {
            cudaGraphExecDestroy(bgraph_exec_);
            bgraph_exec_ = nullptr;
        }
        cudaGraph_t g = nullptr;
        const unsigned long long before = launch_count();
        CG_CUDA(cudaStreamBeginCapture(stream_, cudaStreamCaptureModeThreadLocal));
        try {
            batch_launch(d_x, d_scores);
        } catch (...) {
            cudaStreamEndCapture(stream_, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        CG_CUDA(cudaStreamEndCapture(stream_, &g));
        bgraph_kernels_ = launch_count() - before;  // captured, not launched
        uncount_launches(bgraph_kernels_);
        const cudaError_t ie = cudaGraphInstantiate(&bgraph_exec_, g, 0);
        cudaGraphDestroy(g);
        CG_CUDA(ie);
        bgraph_valid_ = true;
        bgraph_x_ = d_x;
        bgraph_scores_ = d_scores;
        bgraph_stream_ = stream_;
    }
    CG_CUDA(cudaGraphLaunch(bgraph_exec_, stream_));
    count_launches(bgraph_kernels_);
}

void Engine::lof_batched_host(int num, const int64_t* offsets, const int* ks, const float* x, int d, bool normalize,
                              float* scores) {
    if (!x || !scores) throw Error(kInvalidArgument, "points and scores must not be null");
    if (num < 1 || !offsets) throw Error(kInvalidArgument, "num_problems must be >= 1");
    CG_CUDA(cudaSetDevice(device_));
    const int64_t ntot = offsets[num];
    if (ntot < 0) throw Error(kInvalidArgument, "offsets must be non-decreasing");
    float* dx = x_.as<float>(static_cast<size_t>(ntot) * (d > 0 ? d : 1));
    float* ds = scores_.as<float>(static_cast<size_t>(ntot > 0 ? ntot : 1));
    CG_CUDA(cudaMemcpyAsync(dx, x, sizeof(float) * ntot * d, cudaMemcpyHostToDevice, stream_));
    lof_batched_device(num, offsets, ks, dx, d, normalize, ds);
    CG_CUDA(cudaMemcpyAsync(scores, ds, sizeof(float) * ntot, cudaMemcpyDeviceToHost, stream_));
    check_status();
}

}  // namespace culof_gb300

namespace culof_gb300 {
void Engine::batched_tuning(float* ms4, int* per_sm, int* pairs_per_lane) const {
    for (int i = 0; i < 4; ++i) ms4[i] = btuned_ ? btune_ms_[i] : -1.0f;
    const int sms = bbest_grid_ > 0 ? bbest_grid_ : 1;
    int dev_sms = 152;
    cudaDeviceGetAttribute(&dev_sms, cudaDevAttrMultiProcessorCount, device_);
    *per_sm = btuned_ ? sms / (dev_sms > 0 ? dev_sms : 1) : 0;
    *pairs_per_lane = btuned_ ? (bbest_packed_ ? 2 : 1) : 0;
}
}  // namespace culof_gb300
