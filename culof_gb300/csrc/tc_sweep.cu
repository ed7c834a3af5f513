// The fused distance + filtered exact select on the tensor cores
// (8 < d <= 128): the same algorithm as the FP32 sweeps (fast.cu, wide.cu),
// with the per-pair filter value taken from an FP16 Gram tile computed by
// tcgen05.mma instead of an FP32 FMA chain.
//
//   * operands: the centred points in Morton order, scaled by a power of two
//     2^S (so the largest coordinate lands in [2^14, 2^15)) and rounded to
//     f16, row-major [padded][Kp] (Kp = 64 or 128, zero padded);
//   * a CTA owns a 128-row tile (its A operand stays in shared memory) and
//     streams 128-column tiles of the same array by TMA (two stages);
//   * one warp issues the TMA loads, one issues tcgen05.mma (M = N = 128,
//     K = 16 per instruction) into one of two TMEM accumulators, and four
//     epilogue warps read the accumulator back (thread = row), evaluate
//     f = |b|^2 - 2 a.b with packed fma.rn.f32x2 and compare it with the
//     row's threshold tau (sign of a packed subtract);
//   * a passing pair's (f, column) enters the row's list directly (the
//     row's own thread appends it; no global memory is read). Lists are
//     compacted by f: with fk the k-th smallest f in the list, every entry
//     above a proven margin over fk (approx_thr) is strictly farther than
//     k listed columns and is dropped, and the filter threshold tightens to
//     that margin;
//   * at the end each row's surviving entries (about k) are rescored exactly
//     from FP32 row-major coordinates (the oracle's direct-difference chain;
//     coalesced column loads, differences staged in the freed operand
//     buffers) and reduced to the exact k best keys, which the merge of the
//     FP32 sweeps combines with the seed list. A row whose list would
//     overflow with entries inside the margin (heavy duplicates) switches to
//     exact lists: its candidates are then rescored as they pass.
//
// Exactness: the thresholds (row_bounds below) cover the f16 rounding of
// both operands (relative 2^-11, absolute 2^-14 in scaled units for values
// that fall below the f16 normal range or are flushed), the f32 accumulation
// of the tensor core (taken as K * 2^-20 relative), the float32 norms and
// the float32 evaluation of f, so no column that belongs to a row's k
// nearest is ever dropped. Data whose scale cannot be brought into the f16
// range (|S| > 62, or non-finite values) disable the filter: every pair is
// then rescored exactly.
#include <cuda_fp16.h>

#include <cstdlib>

#include "common.cuh"
#include "engine.cuh"
#include "fast.cuh"
#include "sweep_common.cuh"
#include "tc.cuh"

namespace culof_gb300 {

namespace {

using namespace sweep;

constexpr int kTcStages = 2;
constexpr int kEpiWarps = 4;
constexpr int kTcThreads = 32 * (2 + kEpiWarps);  // producer, MMA, 4 epilogue warps
constexpr int kTcQueue = 32 + 32 * 32;            // a drain chunk + one 32-column chunk of every lane
constexpr int kTcM = 128;                         // list capacity per row (k <= 64)
constexpr int kBox = 128 * 128;                   // bytes of one TMA box: 128 rows x 64 f16
constexpr int kTmemCols = 256;                    // two 128-column f32 accumulators

// Scale record on the device: sc = 2^S, k2 = -2 * 2^-2S (undoes the scale of
// a Gram value and doubles it), eta = 2^-14 * 2^-S (absolute f16 rounding
// bound in unscaled units), all = 1 when the filter is disabled.
struct TcScale {
    float sc, k2, eta, all;
};

__device__ __forceinline__ float unflip(unsigned k) {
    return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

// One thread: the scale exponent from the per-dimension min/max keys of the
// spatial-order pass.
__global__ void tc_scale_kernel(const unsigned* __restrict__ mm, int d, TcScale* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    float mx = 0.0f;
    bool finite = true;
    for (int f = 0; f < d; ++f) {
        const float lo = unflip(mm[2 * f]), hi = unflip(mm[2 * f + 1]);
        finite = finite && isfinite(lo) && isfinite(hi);
        mx = fmaxf(mx, fmaxf(fabsf(lo), fabsf(hi)));
    }
    int S = 0;
    bool all = !finite;
    if (finite && mx > 0.0f) {
        S = 14 - ilogbf(mx);
        if (S > 62 || S < -62) all = true;
    }
    if (all) S = 0;
    TcScale r;
    r.sc = ldexpf(1.0f, S);
    r.k2 = -ldexpf(1.0f, 1 - 2 * S);
    r.eta = ldexpf(1.0f, -14 - S);
    r.all = all ? 1.0f : 0.0f;
    *out = r;
}

// Sorted position p: f16 operand row (scaled), FP32 coordinates (row-major,
// dr = d rounded up to 4, zero padded), norm (+inf for padding) and original
// index (kNoIndex for padding). With split, element f < 3d of the row
// operand xh is [hi, lo, hi][f / d] of coordinate f % d and of the column
// operand xb [hi, hi, lo][f / d]; hi = f16(x), lo = f16(x - hi) (x - hi is
// exact in float32).
__global__ void tc_build_kernel(const float* __restrict__ xc, const float* __restrict__ norms, int64_t n, int d,
                                int Kp, int dr, int split, const unsigned* __restrict__ perm, int64_t padded,
                                const TcScale* __restrict__ scale, __half* __restrict__ xh, __half* __restrict__ xb,
                                float* __restrict__ xr, float* __restrict__ cn, unsigned* __restrict__ ix) {
    const float sc = scale->sc;
    const int64_t total = padded * Kp;
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t p = e / Kp;
        const int f = static_cast<int>(e % Kp);
        const bool valid = p < n;
        const unsigned orig = valid ? perm[p] : kNoIndex;
        const int seg = split ? f / d : 0, j = split ? f % d : f;
        const float x = (valid && j < d && seg < 3) ? xc[static_cast<int64_t>(orig) * d + j] : 0.0f;
        const float xs = x * sc;
        const __half hi = __float2half_rn(xs);
        if (split) {
            const __half lo = __float2half_rn(__fsub_rn(xs, __half2float(hi)));
            xh[e] = seg == 1 ? lo : hi;
            xb[e] = seg == 2 ? lo : hi;
        } else {
            xh[e] = hi;
        }
        if (f < dr) xr[p * dr + f] = f < d && valid ? xc[static_cast<int64_t>(orig) * d + f] : 0.0f;
        if (f == 0) {
            cn[p] = valid ? norms[orig] : __int_as_float(0x7f800000);
            ix[p] = orig;
        }
    }
}

// Per row of tile T: the exact k best keys over the tile's own columns and
// the row's starting shared k-th key (as the FP32 seed kernels).
__global__ void __launch_bounds__(256) tc_seed_kernel(const float* __restrict__ xr, const unsigned* __restrict__ ix,
                                                      int t0, int d, int dr, int k, uint64_t* __restrict__ seed_keys,
                                                      unsigned long long* __restrict__ kth_shared) {
    extern __shared__ float spts[];  // [kCT][dr + 1]
    const int T = t0 + static_cast<int>(blockIdx.x);
    const int ld = dr + 1;  // odd stride: lanes reading different points hit different banks
    const int64_t base = static_cast<int64_t>(T) * kCT;
    for (int i = threadIdx.x; i < kCT * dr; i += blockDim.x) {
        const int c = i / dr, f = i % dr;
        spts[c * ld + f] = xr[(base + c) * dr + f];
    }
    unsigned* idx = reinterpret_cast<unsigned*>(spts + kCT * ld);
    for (int i = threadIdx.x; i < kCT; i += blockDim.x) idx[i] = ix[base + i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int r = warp; r < kRT; r += nw) {
        const int64_t pos = base + r;
        const bool row_valid = idx[r] != kNoIndex;
        // the lane's four columns as four independent chains (each in the
        // oracle's order), the row's coordinate loaded once per dimension
        float s4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
        for (int f = 0; f < d; ++f) {
            const float a = spts[r * ld + f];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float t = __fsub_rn(a, spts[(j * 32 + lane) * ld + f]);
                s4[j] = __fmaf_rn(t, t, s4[j]);
            }
        }
        uint64_t v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = j * 32 + lane;
            v[j] = (row_valid && c != r && idx[c] != kNoIndex) ? make_key(__float_as_uint(s4[j]), idx[c]) : kKeyMax;
        }
        warp_bitonic_sort<4>(v);
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int e = j * 32 + lane;
            if (e < k) seed_keys[pos * k + e] = v[j];
        }
        const int owner = (k - 1) & 31, oreg = (k - 1) >> 5;
        uint64_t kk = kKeyMax;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const uint64_t t = __shfl_sync(0xffffffffu, v[j], owner);
            if (j == oreg) kk = t;
        }
        if (lane == 0) kth_shared[pos] = row_valid ? kk : kKeyMax;
    }
}

// ---- thresholds ---------------------------------------------------------------
// Per row a (float32 norm na, K = Kp terms, u = 2^-24, g the relative error of
// the float32 norms, A >= |a|, B >= |b| for every column b), the f16 Gram value
// G of a column b and its filter value f = fl(Nb - 2 G) satisfy
//   |G - a.b| <= E = (2 uh + uh^2) A B + eta (1 + uh) sqrt(K) (A + B) + K eta^2
//                    + K ua ((1 + uh) A + sqrt(K) eta) ((1 + uh) B + sqrt(K) eta)
//   |f - (|b|^2 - 2 a.b)| <= m0 = g / (1 - g) Nmax + 2 E + u (Nmax + 2 (A B + E))
// (uh = 2^-11 the f16 rounding, eta the absolute f16 error, ua = 2^-20 per
// accumulated term of the tensor core). Two consequences, each evaluated with
// upward rounding:
//  * exact threshold: a column whose exact float32 distance is <= D has
//    f <= D c1 + c0 (c1 = (1 + 8u) / (1 - (K + 2) u),
//    c0 = -na / (1 + g) + m0 + 8u (na + Nmax + 2 A B));
//  * approximate threshold: with T the real squared distance and
//    D in T [1 - dl, 1 + dl] (dl = (K + 3) u / (1 - (K + 3) u)), a column b with
//    f_b > thr(fk) = fk + 2 m0 + 2 dl / (1 - dl) max(0, fk + na / (1 - g) + m0)
//    (+ slack) is strictly farther than every column c with f_c <= fk, so once
//    k columns with f <= fk are known, b can never be among the k nearest.
// With split operands (x = hi + r exactly, lo = f16(r), |r| <= uh |x|,
// |lo - r| <= uh |r| + eta) the summed products hi.hi + lo.hi + hi.lo miss
// a.b by at most
//   E = (3 uh^2 + 3 uh^3) A B + eta (1 + uh) sqrt(d) (A + B) + 2 d eta^2
//       + Ka ua (1 + 3 uh) ((1 + uh) A + sqrt(Ka) eta) ((1 + uh) B + sqrt(Ka) eta)
// (Ka = the accumulated K, 16 per MMA step), in place of the first line of E.
struct RowBounds {
    float c0, c3, c4;  // per row: exact offset; approximate offset and shift
};
constexpr double kU = 5.9604644775390625e-08;  // 2^-24

__device__ RowBounds row_bounds(float na_f, float nmax_f, int K, float eta_f, int split_d, int kacc) {
    const double uh = 4.8828125e-04;        // 2^-11
    const double ua = 9.5367431640625e-07;  // 2^-20
    const double g = (K + 1) * kU / (1.0 - (K + 1) * kU);
    const double a = static_cast<double>(na_f), m = static_cast<double>(nmax_f), eta = static_cast<double>(eta_f);
    const double A = sqrt(a / (1.0 - g)), B = sqrt(m / (1.0 - g));
    double E;
    if (split_d > 0) {
        const double sd = sqrt(static_cast<double>(split_d)), sa = sqrt(static_cast<double>(kacc));
        E = (3.0 * uh * uh + 3.0 * uh * uh * uh) * A * B + eta * (1.0 + uh) * sd * (A + B) +
            2.0 * split_d * eta * eta +
            kacc * ua * (1.0 + 3.0 * uh) * ((1.0 + uh) * A + sa * eta) * ((1.0 + uh) * B + sa * eta);
    } else {
        const double sk = sqrt(static_cast<double>(K));
        E = (2.0 * uh + uh * uh) * A * B + eta * (1.0 + uh) * sk * (A + B) + K * eta * eta +
            K * ua * ((1.0 + uh) * A + sk * eta) * ((1.0 + uh) * B + sk * eta);
    }
    const double m0 = g / (1.0 - g) * m + 2.0 * E + kU * (m + 2.0 * (A * B + E));
    const double slack = 8.0 * kU * (a + m + 2.0 * A * B) + 1e-30;
    RowBounds r;
    r.c0 = __double2float_ru(-a / (1.0 + g) + m0 + slack);
    r.c3 = __double2float_ru(2.0 * m0 + slack);
    r.c4 = __double2float_ru(a / (1.0 - g) + m0);
    return r;
}
__device__ __forceinline__ float exact_c1(int K) {
    return __double2float_ru((1.0 + 8.0 * kU) / (1.0 - (K + 2) * kU));
}
__device__ __forceinline__ float approx_c2(int K) {
    const double dl = (K + 3) * kU / (1.0 - (K + 3) * kU);
    return __double2float_ru(2.0 * dl / (1.0 - dl) * (1.0 + 8.0 * kU));
}
// Filter threshold of a row from its exact k-th key.
__device__ __forceinline__ float exact_tau(uint64_t kth, float c1, float c0) {
    if (kth == kKeyMax) return __int_as_float(0x7f800000);
    return __fmaf_ru(__uint_as_float(key_bits(kth)), c1, c0);
}
// The approximate threshold over a k-th filter value fk.
__device__ __forceinline__ float approx_thr(float fk, float c2, float c3, float c4) {
    return __fadd_ru(fk, __fmaf_ru(fmaxf(0.0f, __fadd_ru(fk, c4)), c2, c3));
}

__device__ __forceinline__ uint64_t tau_pair(float tau) {
    // f <= tau  <=>  f - next_up(tau) < 0 (the sign of a rounded difference
    // is exact), so a packed subtract's sign bits decide two columns at once.
    const float t = isinf(tau) ? tau : nextafterf(tau, __int_as_float(0x7f800000));
    return dup2(t);
}

__device__ __forceinline__ uint64_t sub2(uint64_t a, uint64_t b) {
    uint64_t d;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(a), "l"(b));
    return d;
}
__device__ __forceinline__ uint64_t pack2(float lo, float hi) {
    return static_cast<uint64_t>(__float_as_uint(lo)) | (static_cast<uint64_t>(__float_as_uint(hi)) << 32);
}
__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Order-preserving bits of a float (negative values included).
__device__ __forceinline__ uint32_t flip_bits(float f) {
    const uint32_t u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// Row modes: approximate lists hold (flip(f) << 32 | sorted column position);
// exact lists hold the usual (distance bits << 32 | original index).
constexpr int kModeApprox = 0;
constexpr int kModeExact = 1;

// Per-row lists live in global memory (L2-resident while their CTA runs):
// kTcM keys per row, 128 rows per CTA. Keeping them out of shared memory
// lets two CTAs share an SM, so two epilogue warps per SM sub-partition
// hide each other's latencies.
constexpr int kTcListRow = kTcM;
constexpr size_t kTcListCta = static_cast<size_t>(kRT) * kTcListRow;  // keys per CTA
constexpr int kTcMaxCtasPerLaunch = 4096;                             // bounds the list workspace (512 MiB)

struct TcSmem {
    uint8_t a[2][kBox];             // row tile operand (K boxes 0..1)
    uint8_t b[kTcStages][2][kBox];  // column tile operands
    uint64_t kth[kRT];              // exact k-th key known for the row (only decreases)
    float athr[kRT];                // approximate threshold of the row's list (+inf until k entries)
    float row_norm[kRT];
    int cnt[kRT];
    int sorted[kRT];  // the row's list[0..sorted) is sorted (the last compaction's result)
    int mode[kRT];
    uint16_t queue[kEpiWarps][kTcQueue];  // exact-mode candidates (row << 8 | column) of the current tile
    float nb[kEpiWarps][2][kCT];          // column norms of the current and the next tile, per epilogue warp
    uint64_t full[kTcStages], empty[kTcStages], tfull[2], tempty[2], afull, fin;
    uint32_t tmem_base;
    int abort;
};
static_assert(2 * (sizeof(TcSmem) + 1024 + 1024) <= 233472, "two tensor-sweep CTAs must fit on an SM");
// The final exact rescoring reuses the operand buffers (free once the last MMA
// has completed): per epilogue warp, 32 candidates x (128 + 1) differences.
constexpr int kScratchLd = 129;
static_assert(kEpiWarps * 32 * kScratchLd * 4 <= 3 * 2 * kBox, "scratch fits in the operand buffers");

__device__ void tc_abort(TcSmem& sh, int* status) {
    *reinterpret_cast<volatile int*>(&sh.abort) = 1;
    atomicExch(status, 1);
}
__device__ __forceinline__ bool tc_aborted(TcSmem& sh) { return *reinterpret_cast<volatile int*>(&sh.abort) != 0; }

// g[b] for a lane-dependent b, without local memory: a 5-level select tree.
__device__ __forceinline__ uint32_t select32(const uint32_t (&g)[32], int b) {
    uint32_t v16[16], v8[8], v4[4], v2[2];
#pragma unroll
    for (int i = 0; i < 16; ++i) v16[i] = (b & 16) ? g[16 + i] : g[i];
#pragma unroll
    for (int i = 0; i < 8; ++i) v8[i] = (b & 8) ? v16[8 + i] : v16[i];
#pragma unroll
    for (int i = 0; i < 4; ++i) v4[i] = (b & 4) ? v8[4 + i] : v8[i];
#pragma unroll
    for (int i = 0; i < 2; ++i) v2[i] = (b & 2) ? v4[2 + i] : v4[i];
    return (b & 1) ? v2[1] : v2[0];
}

// Exact key of (row position pa, column position pb), one lane: the oracle's
// direct-difference chain over row-major FP32 coordinates.
__device__ __forceinline__ uint64_t exact_key_lane(const float* __restrict__ xr, const unsigned* __restrict__ ix,
                                                   int64_t pa, int64_t pb, int d, int dr) {
    const unsigned ib = __ldg(ix + pb);
    if (ib == kNoIndex) return kKeyMax;
    const float4* va = reinterpret_cast<const float4*>(xr + pa * dr);
    const float4* vb = reinterpret_cast<const float4*>(xr + pb * dr);
    float s = 0.0f;
    for (int f4 = 0; 4 * f4 < d; ++f4) {
        const float4 x = __ldg(va + f4), y = __ldg(vb + f4);
        const float xa[4] = {x.x, x.y, x.z, x.w}, yb[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            if (4 * f4 + q < d) {
                const float t = __fsub_rn(xa[q], yb[q]);
                s = __fmaf_rn(t, t, s);
            }
        }
    }
    return make_key(__float_as_uint(s), ib);
}

constexpr int kListE = kTcListRow / 32;  // list keys per lane in a compaction
static_assert(kListE == 4, "the compaction sorts 4 keys per lane");

// Exact list of row r (whole warp): sort, drop duplicates, keep the k
// smallest; tighten the row's exact k-th key.
__noinline__ __device__ void compact_exact(TcSmem& sh, uint64_t* __restrict__ lst, int r, int k) {
    const int lane = threadIdx.x & 31;
    const int c = min(sh.cnt[r], kTcListRow);
    {
        const int s = sh.sorted[r];
        if (s <= c && c - s <= 64) {  // merge the new entries into the sorted prefix
            uint64_t kk;
            const int kept = merge_sorted_prefix(lst, s, c, k, k - 1, [](uint64_t) { return kKeyMax; }, &kk);
            if (lane == 0) {
                sh.cnt[r] = kept;
                sh.sorted[r] = kept;
                if (kk != kKeyMax && kk < sh.kth[r]) sh.kth[r] = kk;
            }
            __syncwarp();
            return;
        }
    }
    uint64_t v[kListE];
#pragma unroll
    for (int j = 0; j < kListE; ++j) {
        const int e = j * 32 + lane;
        v[j] = e < c ? lst[e] : kKeyMax;
    }
    warp_bitonic_sort<kListE>(v);
    int rank[kListE];
    const int uniq = warp_unique_ranks<kListE>(v, kKeyMax, rank);
    __syncwarp();
    uint64_t kth_new = kKeyMax;
#pragma unroll
    for (int j = 0; j < kListE; ++j) {
        if (rank[j] >= 0 && rank[j] < k) lst[rank[j]] = v[j];
        if (rank[j] == k - 1) kth_new = v[j];
    }
    const unsigned m = __ballot_sync(0xffffffffu, kth_new != kKeyMax);
    const uint64_t kk = __shfl_sync(0xffffffffu, kth_new, m ? __ffs(m) - 1 : 0);
    if (lane == 0) {
        sh.cnt[r] = min(uniq, k);
        sh.sorted[r] = min(uniq, k);
        if (m && kk < sh.kth[r]) sh.kth[r] = kk;
    }
    __syncwarp();
}

// Sort row r's approximate list (whole warp), find its k-th filter value fk
// and keep the entries with f <= approx_thr(fk) (all of them while fewer than
// k are known). Returns the number kept; if that exceeds `cap`, the list is
// left untrimmed and the caller decides.
__noinline__ __device__ int approx_compact(TcSmem& sh, uint64_t* __restrict__ lst, int r, int k, float c2, float c3,
                                           float c4, int cap) {
    const int lane = threadIdx.x & 31;
    const int c = min(sh.cnt[r], kTcListRow);
    {
        const int s = sh.sorted[r];
        if (s <= c && c - s <= 64) {  // merge the new entries into the sorted prefix
            float thr = __int_as_float(0x7f800000);
            uint64_t fk;
            // entries above the margin over the k-th value are dropped (fewer
            // than k entries: all are kept)
            const int keep = merge_sorted_prefix(
                lst, s, c, kTcListRow, k - 1,
                [&](uint64_t key) -> uint64_t {
                    if (key == kKeyMax) return kKeyMax;
                    thr = approx_thr(unflip(key_bits(key)), c2, c3, c4);
                    return (static_cast<uint64_t>(flip_bits(thr)) << 32) | 0xFFFFFFFFull;
                },
                &fk);
            if (lane == 0) {
                sh.cnt[r] = keep;
                sh.sorted[r] = keep;
                if (keep <= cap) sh.athr[r] = thr;
            }
            __syncwarp();
            return keep;
        }
    }
    uint64_t v[kListE];
#pragma unroll
    for (int j = 0; j < kListE; ++j) {
        const int e = j * 32 + lane;
        v[j] = e < c ? lst[e] : kKeyMax;
    }
    warp_bitonic_sort<kListE>(v);
    float thr = __int_as_float(0x7f800000);
    if (c >= k) {
        const int owner = (k - 1) & 31, oreg = (k - 1) >> 5;
        uint64_t kk = kKeyMax;
#pragma unroll
        for (int j = 0; j < kListE; ++j) {
            const uint64_t t = __shfl_sync(0xffffffffu, v[j], owner);
            if (j == oreg) kk = t;
        }
        thr = approx_thr(unflip(key_bits(kk)), c2, c3, c4);
    }
    int keep = 0;
#pragma unroll
    for (int j = 0; j < kListE; ++j) {
        const bool in = v[j] != kKeyMax && unflip(key_bits(v[j])) <= thr;
        keep += __popc(__ballot_sync(0xffffffffu, in));
    }
    if (keep <= cap) {
#pragma unroll
        for (int j = 0; j < kListE; ++j) {
            const int e = j * 32 + lane;
            if (e < keep) lst[e] = v[j];
        }
        if (lane == 0) {
            sh.cnt[r] = keep;
            sh.sorted[r] = keep;
            sh.athr[r] = thr;
        }
    }
    __syncwarp();
    return keep;
}

// Row r leaves approximate mode (its list would overflow with entries within
// the approximate margin, e.g. many duplicates): every entry is rescored
// exactly (one lane per entry) and the list becomes an exact k-best list.
__noinline__ __device__ void to_exact_mode(TcSmem& sh, uint64_t* __restrict__ lst, int r, int64_t rbase,
                                           const float* __restrict__ xr, const unsigned* __restrict__ ix, int d,
                                           int dr, int k) {
    const int lane = threadIdx.x & 31;
    const int c = min(sh.cnt[r], kTcListRow);
    for (int e = lane; e < c; e += 32) {
        const int64_t pb = static_cast<int64_t>(key_index(lst[e]));
        lst[e] = exact_key_lane(xr, ix, rbase + r, pb, d, dr);
    }
    __syncwarp();
    if (lane == 0) {
        sh.mode[r] = kModeExact;
        sh.sorted[r] = 0;  // exact keys: the approximate order no longer holds
    }
    __syncwarp();
    compact_exact(sh, lst, r, k);
}

// Rescore the warp's queued exact-mode pairs of column tile cbase exactly and
// add the keys that beat their row's k-th key. True if a list was compacted.
__noinline__ __device__ bool tc_drain(TcSmem& sh, uint64_t* __restrict__ glist, int wq, int row0, int qc,
                                      int64_t rbase, int64_t cbase, const float* __restrict__ xr,
                                      const unsigned* __restrict__ ix, int d, int dr, int k) {
    const int lane = threadIdx.x & 31;
    bool compacted = false;
    for (int base = 0; base < qc; base += 32) {
        const int i = base + lane;
        if (i < qc) {
            const unsigned e = sh.queue[wq][i];
            const int r = static_cast<int>(e >> 8), c = static_cast<int>(e & 0xFF);
            const uint64_t key = exact_key_lane(xr, ix, rbase + r, cbase + c, d, dr);
            if (key < sh.kth[r]) {
                const int slot = atomicAdd(&sh.cnt[r], 1);
                glist[static_cast<size_t>(r) * kTcListRow + slot] = key;
            }
        }
        __syncwarp();
        unsigned full = __ballot_sync(0xffffffffu,
                                      sh.mode[row0 + lane] == kModeExact && sh.cnt[row0 + lane] > kTcListRow - 32);
        compacted |= full != 0;
        while (full) {
            const int rr = row0 + __ffs(full) - 1;
            full &= full - 1;
            compact_exact(sh, glist + static_cast<size_t>(rr) * kTcListRow, rr, k);
        }
    }
    return compacted;
}

// Final exact rescoring of the first P approximate entries of row r (whole
// warp): lane l loads dimensions 4l..4l+3 of each candidate column with one
// coalesced 512-byte warp load per column, forms the differences t = a - b
// and stages them in shared memory; lane i then runs candidate i's FMA chain
// in dimension order (bit-identical to the oracle's formula).
__noinline__ __device__ void rescore_final(uint64_t* __restrict__ lst, int r, int P, float* __restrict__ scratch,
                                           int64_t rbase, const float* __restrict__ xr,
                                           const unsigned* __restrict__ ix, int d, int dr) {
    const int lane = threadIdx.x & 31;
    const bool has = 4 * lane < dr;
    const float4 a4 = has ? __ldg(reinterpret_cast<const float4*>(xr + (rbase + r) * dr) + lane)
                          : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int base = 0; base < P; base += 32) {
        const int nb = min(32, P - base);
        const uint32_t mypos = lane < nb ? key_index(lst[base + lane]) : 0u;
        for (int i0 = 0; i0 < nb; i0 += 8) {
            float4 b4[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const int i = i0 + q;
                const uint32_t pb = __shfl_sync(0xffffffffu, mypos, i & 31);
                b4[q] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (i < nb && has) b4[q] = __ldg(reinterpret_cast<const float4*>(xr + static_cast<int64_t>(pb) * dr) + lane);
            }
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                float* t = scratch + (i0 + q) * kScratchLd + 4 * lane;
                if (i0 + q < nb && has) {
                    t[0] = __fsub_rn(a4.x, b4[q].x);
                    t[1] = __fsub_rn(a4.y, b4[q].y);
                    t[2] = __fsub_rn(a4.z, b4[q].z);
                    t[3] = __fsub_rn(a4.w, b4[q].w);
                }
            }
        }
        __syncwarp();
        uint64_t key = kKeyMax;
        if (lane < nb) {
            const unsigned ib = __ldg(ix + mypos);
            if (ib != kNoIndex) {
                const float* t = scratch + lane * kScratchLd;
                float s = 0.0f;
                for (int f = 0; f < d; ++f) s = __fmaf_rn(t[f], t[f], s);
                key = make_key(__float_as_uint(s), ib);
            }
        }
        __syncwarp();
        if (lane < nb) lst[base + lane] = key;
        __syncwarp();
    }
}

__global__ void __launch_bounds__(kTcThreads, 2)
tc_sweep_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ CUtensorMap tmapb,
                const float* __restrict__ xr,
                const float* __restrict__ cn, const unsigned* __restrict__ ix, const TcScale* __restrict__ scale,
                int nt, int T0, int ntb, int nsplit, int d, int dr, int Kp, int split_ops, int ksteps, int k,
                const unsigned* __restrict__ max_norm_bits, unsigned long long* __restrict__ kth_shared,
                uint64_t* __restrict__ partial, uint64_t* __restrict__ lists, int* __restrict__ status, int qs,
                const uint2* __restrict__ plist, const int* __restrict__ pcount) {
    extern __shared__ uint8_t tc_raw[];
    TcSmem& sh = *reinterpret_cast<TcSmem*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int T = T0 + static_cast<int>(blockIdx.x) % ntb;
    const int split = static_cast<int>(blockIdx.x) / ntb;
    // the split's column tiles: entries split + nsplit j of the row tile's
    // prune list (visiting order, tiles that the seed's k-th distances cannot
    // rule out), or its contiguous share of the spiral past the seed window
    const int per = (nt - qs + nsplit - 1) / nsplit;
    const int q0 = qs + split * per;
    const int q1 = min(nt, q0 + per);
    const int lcount = plist ? pcount[T] : 0;
    const int count = plist ? (lcount > split ? (lcount - split + nsplit - 1) / nsplit : 0) : (q1 > q0 ? q1 - q0 : 0);
    const uint2* tlist = plist ? plist + static_cast<int64_t>(T) * nt : nullptr;
    auto col_tile = [&](int j) -> int {
        return tlist ? static_cast<int>(tlist[split + nsplit * j].x) : spiral_tile(T, q0 + j, nt);
    };
    const int nkb = Kp / 64;
    const float nmax = __uint_as_float(*max_norm_bits);
    const int64_t rbase = static_cast<int64_t>(T) * kRT;
    uint64_t* glist = lists + static_cast<size_t>(blockIdx.x) * kTcListCta;

    if (tid == 0) {
        for (int s = 0; s < kTcStages; ++s) {
            mbar_init(&sh.full[s], 1);
            mbar_init(&sh.empty[s], 1);
        }
        for (int a = 0; a < 2; ++a) {
            mbar_init(&sh.tfull[a], 1);
            mbar_init(&sh.tempty[a], kEpiWarps);
        }
        mbar_init(&sh.afull, 1);
        mbar_init(&sh.fin, 1);
        sh.abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) tc::tmem_alloc(&sh.tmem_base, kTmemCols);
    if (warp >= 2) {
        const int r = 32 * (warp & 3) + lane;
        sh.kth[r] = kth_shared[rbase + r];
        sh.row_norm[r] = cn[rbase + r];
        sh.cnt[r] = 0;
        sh.sorted[r] = 0;
        sh.athr[r] = __int_as_float(0x7f800000);
        // with the filter disabled the f values carry no information: exact lists
        sh.mode[r] = scale->all != 0.0f ? kModeExact : kModeApprox;
    }
    tc::tc_fence_before();
    __syncthreads();
    tc::tc_fence_after();
    const uint32_t tmem = sh.tmem_base;

    if (warp == 0) {
        // ---- TMA producer
        if (lane == 0) {
            int issued = 0;
            mbar_expect_tx(&sh.afull, nkb * kBox);
            for (int kb = 0; kb < nkb; ++kb) tc::tma_load_2d(sh.a[kb], &tmap, 64 * kb, static_cast<int>(rbase), &sh.afull);
            for (int j = 0; j < count; ++j) {
                const int s = j & 1;
                if (j >= kTcStages && !mbar_wait(&sh.empty[s], ((j >> 1) - 1) & 1)) {
                    tc_abort(sh, status);
                    break;
                }
                if (tc_aborted(sh)) break;
                const int col0 = col_tile(j) * kCT;
                mbar_expect_tx(&sh.full[s], nkb * kBox);
                for (int kb = 0; kb < nkb; ++kb) tc::tma_load_2d(sh.b[s][kb], &tmapb, 64 * kb, col0, &sh.full[s]);
                issued = j + 1;
            }
            // no copy may still be landing in shared memory when the CTA exits
            if (!mbar_wait(&sh.afull, 0)) atomicExch(status, 1);
            for (int j = issued - kTcStages; j < issued; ++j)
                if (j >= 0 && !mbar_wait(&sh.full[j & 1], (j >> 1) & 1)) atomicExch(status, 1);
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---- MMA issuer
        if (lane == 0) {
            constexpr uint32_t idesc = tc::f16_idesc(128, 128);
            bool ok = mbar_wait(&sh.afull, 0);
            if (!ok) tc_abort(sh, status);
            for (int j = 0; ok && j < count; ++j) {
                const int s = j & 1, acc = j & 1;
                if (tc_aborted(sh) || !mbar_wait(&sh.full[s], (j >> 1) & 1) ||
                    (j >= 2 && !mbar_wait(&sh.tempty[acc], ((j >> 1) - 1) & 1))) {
                    tc_abort(sh, status);
                    break;
                }
                tc::tc_fence_after();
                const uint32_t dt = tmem + static_cast<uint32_t>(acc * 128);
                for (int kk = 0; kk < ksteps; ++kk) {
                    const int kb = kk >> 2, sub = kk & 3;
                    const uint64_t ad = tc::sw128_desc(smem_u32(sh.a[kb]) + 32 * sub);
                    const uint64_t bd = tc::sw128_desc(smem_u32(sh.b[s][kb]) + 32 * sub);
                    tc::mma_f16kind(dt, ad, bd, idesc, kk > 0);
                }
                tc::mma_commit(&sh.empty[s]);
                tc::mma_commit(&sh.tfull[acc]);
            }
            // every MMA issued has completed before TMEM is released
            tc::mma_commit(&sh.fin);
            if (!mbar_wait(&sh.fin, 0)) atomicExch(status, 1);
        }
        __syncwarp();
    } else {
        // ---- epilogue: thread = row
        const int wq = warp - 2;
        const int row0 = 32 * (warp & 3);
        const int r = row0 + lane;
        uint64_t* const mylist = glist + static_cast<size_t>(r) * kTcListRow;
        const TcScale sc = *scale;
        const bool all = sc.all != 0.0f;
        const bool row_valid = __ldg(ix + rbase + r) != kNoIndex;
        const RowBounds rb = row_bounds(sh.row_norm[r], nmax, Kp, sc.eta, split_ops ? d : 0, 16 * ksteps);
        const float c1 = exact_c1(Kp), c2 = approx_c2(Kp);
        auto row_tau = [&]() -> float {
            if (!row_valid) return __int_as_float(0xff800000);
            float t = exact_tau(sh.kth[r], c1, rb.c0);
            if (sh.mode[r] == kModeApprox) t = fminf(t, sh.athr[r]);
            return t;
        };
        uint64_t tq = tau_pair(row_tau());
        const uint64_t k2 = dup2(sc.k2);
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(row0) << 16);
        // This tile's column norms are staged in a per-warp shared ring one
        // tile ahead (one coalesced 512-byte load per warp), so the filter
        // never waits on global memory.
        auto tile_base = [&](int jj) -> int64_t { return static_cast<int64_t>(col_tile(jj)) * kCT; };
        float4 npre = make_float4(0.f, 0.f, 0.f, 0.f);
        if (count > 0) npre = __ldg(reinterpret_cast<const float4*>(cn + tile_base(0)) + lane);
        int qc = 0;
        int64_t cbase = 0;
        const float* nbj = nullptr;
        // filter one 32-column chunk held in registers; list / queue its candidates
        auto process_chunk = [&](const uint32_t (&gr)[32], int ch) {
            uint64_t dl[16];
            unsigned signs = 0;
            const float4* nb4 = reinterpret_cast<const float4*>(nbj + 32 * ch);
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                const float4 nb = nb4[q];
                const uint64_t f0 = fma2(pack2(__uint_as_float(gr[4 * q]), __uint_as_float(gr[4 * q + 1])), k2,
                                         pack2(nb.x, nb.y));
                const uint64_t f1 = fma2(pack2(__uint_as_float(gr[4 * q + 2]), __uint_as_float(gr[4 * q + 3])), k2,
                                         pack2(nb.z, nb.w));
                dl[2 * q] = sub2(f0, tq);
                dl[2 * q + 1] = sub2(f1, tq);
                signs |= static_cast<unsigned>(dl[2 * q]) | static_cast<unsigned>(dl[2 * q] >> 32) |
                         static_cast<unsigned>(dl[2 * q + 1]) | static_cast<unsigned>(dl[2 * q + 1] >> 32);
            }
            if (all) signs = row_valid ? 0x80000000u : 0u;
            if (!__any_sync(0xffffffffu, static_cast<int>(signs) < 0)) return;
            unsigned pass = 0;
            if (all) {
                pass = row_valid ? 0xFFFFFFFFu : 0u;
            } else {
#pragma unroll
                for (int q = 0; q < 16; ++q) {
                    pass |= (static_cast<unsigned>(dl[q]) >> 31) << (2 * q);
                    pass |= static_cast<unsigned>(dl[q] >> 63) << (2 * q + 1);
                }
            }
            const bool exact_row = sh.mode[r] == kModeExact;
            if (!exact_row && pass) {
                // approximate keys straight into the row's own list (f
                // recomputed exactly as the packed filter did)
                int cnt = sh.cnt[r];
                unsigned pp = pass;
                while (pp) {
                    const int b = __ffs(pp) - 1;
                    pp &= pp - 1;
                    const float f = __fmaf_rn(__uint_as_float(select32(gr, b)), sc.k2, nbj[32 * ch + b]);
                    mylist[cnt++] = make_key(flip_bits(f), static_cast<uint32_t>(cbase + 32 * ch + b));
                }
                sh.cnt[r] = cnt;
            }
            if (__any_sync(0xffffffffu, exact_row && pass)) {
                int tot;
                int off = warp_prefix_offset(exact_row ? __popc(pass) : 0, tot);
                if (exact_row) {
                    unsigned pp = pass;
                    while (pp) {
                        const int b = __ffs(pp) - 1;
                        pp &= pp - 1;
                        sh.queue[wq][qc + off++] = static_cast<uint16_t>((r << 8) | (32 * ch + b));
                    }
                }
                qc += tot;
            }
            __syncwarp();
            // keep room for the next chunk: compact approximate lists with
            // less than 32 free slots
            unsigned full =
                __ballot_sync(0xffffffffu, sh.mode[r] == kModeApprox && sh.cnt[r] > kTcListRow - 32);
            bool changed = full != 0;
            while (full) {
                const int src = __ffs(full) - 1;
                full &= full - 1;
                const int rr = row0 + src;
                uint64_t* lst = glist + static_cast<size_t>(rr) * kTcListRow;
                const float c3 = __shfl_sync(0xffffffffu, rb.c3, src);
                const float c4 = __shfl_sync(0xffffffffu, rb.c4, src);
                if (approx_compact(sh, lst, rr, k, c2, c3, c4, kTcListRow - 32) > kTcListRow - 32)
                    to_exact_mode(sh, lst, rr, rbase, xr, ix, d, dr, k);
            }
            if (qc >= 32) {
                changed |= tc_drain(sh, glist, wq, row0, qc, rbase, cbase, xr, ix, d, dr, k);
                qc = 0;
            }
            if (changed) tq = tau_pair(row_tau());
        };
        for (int j = 0; j < count; ++j) {
            const int acc = j & 1;
            cbase = tile_base(j);
            float* nbw = sh.nb[wq][j & 1];
            reinterpret_cast<float4*>(nbw)[lane] = npre;
            if (j + 1 < count) npre = __ldg(reinterpret_cast<const float4*>(cn + tile_base(j + 1)) + lane);
            nbj = nbw;
            __syncwarp();
            if (!mbar_wait_warp(&sh.tfull[acc], (j >> 1) & 1)) {
                if (lane == 0) tc_abort(sh, status);
                break;
            }
            tc::tc_fence_after();
            qc = 0;
            // one 32-column chunk at a time, one call site: double-buffering
            // the TMEM loads inlines the filter twice and costs more in code
            // size and registers (168 with spills against 128) than the
            // overlap saves (factor-model sweep at n = 200k, d = 128, k = 50:
            // 40.6 ms against 35.0 ms)
            const uint32_t taddr = lane_addr + static_cast<uint32_t>(acc * 128);
            uint32_t ga[32];
#pragma unroll 1
            for (int ch = 0; ch < 4; ++ch) {
                tc::tmem_ld32_async(taddr + static_cast<uint32_t>(32 * ch), ga);
                tc::tmem_wait32(ga);
                process_chunk(ga, ch);
            }
            // the accumulator is free for the next tile but one
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&sh.tempty[acc]);
            if (qc > 0 && tc_drain(sh, glist, wq, row0, qc, rbase, cbase, xr, ix, d, dr, k)) tq = tau_pair(row_tau());
        }
        // ---- final: exact k best of this split per row; share the k-th key.
        // The operand buffers are free once every epilogue warp has read its
        // last accumulator (the MMAs that read them have completed).
        asm volatile("bar.sync 1, %0;" ::"r"(32 * kEpiWarps) : "memory");
        float* scratch = reinterpret_cast<float*>(&sh.a[0][0]) + wq * 32 * kScratchLd;
        for (int i = 0; i < 32; ++i) {
            const int rr = row0 + i;
            uint64_t* lst = glist + static_cast<size_t>(rr) * kTcListRow;
            if (sh.mode[rr] == kModeApprox) {
                const float c3 = __shfl_sync(0xffffffffu, rb.c3, i);
                const float c4 = __shfl_sync(0xffffffffu, rb.c4, i);
                const int P = approx_compact(sh, lst, rr, k, c2, c3, c4, kTcListRow);
                rescore_final(lst, rr, P, scratch, rbase, xr, ix, d, dr);
                if (lane == 0) {
                    sh.mode[rr] = kModeExact;
                    sh.sorted[rr] = 0;  // exact keys: the approximate order no longer holds
                }
                __syncwarp();
            }
            compact_exact(sh, lst, rr, k);
            const int64_t pos = rbase + rr;
            const int c = sh.cnt[rr];
            uint64_t* out = partial + (static_cast<int64_t>(split) * nt * kRT + pos) * k;
            for (int e = lane; e < k; e += 32) out[e] = e < c ? lst[e] : kKeyMax;
            if (lane == 0 && sh.kth[rr] != kKeyMax)
                atomicMin(&kth_shared[pos], static_cast<unsigned long long>(sh.kth[rr]));
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, kTmemCols);
    }
}

}  // namespace

// Split operands when the three d-wide segments fit one or two 64-wide
// boxes (d <= 42). CULOF_TC_SPLIT=0 keeps single f16 operands (measurement).
static bool tc_use_split(int d) {
    const char* env = std::getenv("CULOF_TC_SPLIT");
    if (env && env[0] == '0') return false;
    return 3 * d <= 128;
}
static int tc_kp(int d, bool split) {
    const int w = split ? 3 * d : d;
    return w <= 64 ? 64 : 128;
}

size_t tc_buffer_bytes(int64_t padded, int d) {
    const bool split = tc_use_split(d);
    const int Kp = tc_kp(d, split);
    const int dr = (d + 3) & ~3;
    const auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    return up(sizeof(__half) * padded * Kp) * (split ? 2 : 1) + up(sizeof(float) * padded * dr) +
           up(sizeof(float) * padded) + up(sizeof(unsigned) * padded) + up(sizeof(TcScale));
}

size_t tc_list_bytes(int nt, int nsplit) {
    int64_t ctas = static_cast<int64_t>(nt) * nsplit;
    if (ctas > kTcMaxCtasPerLaunch) ctas = kTcMaxCtasPerLaunch;
    return sizeof(uint64_t) * kTcListCta * static_cast<size_t>(ctas);
}

TcBuffers tc_prepare(void* buf, const float* xc, const float* norms, int64_t n, int d, const unsigned* perm, int nt,
                     const unsigned* minmax, cudaStream_t s) {
    const int64_t padded = static_cast<int64_t>(nt) * kCT;
    const auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    TcBuffers b;
    const bool split = tc_use_split(d);
    b.split = split ? 1 : 0;
    b.Kp = tc_kp(d, split);
    b.ksteps = split ? (3 * d + 15) / 16 : b.Kp / 16;
    b.dr = (d + 3) & ~3;
    char* p = static_cast<char*>(buf);
    b.xh = p;
    p += up(sizeof(__half) * padded * b.Kp);
    b.xb = b.xh;
    if (split) {
        b.xb = p;
        p += up(sizeof(__half) * padded * b.Kp);
    }
    b.xr = reinterpret_cast<float*>(p);
    p += up(sizeof(float) * padded * b.dr);
    b.cn = reinterpret_cast<float*>(p);
    p += up(sizeof(float) * padded);
    b.ix = reinterpret_cast<unsigned*>(p);
    p += up(sizeof(unsigned) * padded);
    b.scale = p;
    tc_scale_kernel<<<1, 32, 0, s>>>(minmax, d, reinterpret_cast<TcScale*>(b.scale));
    CG_LAUNCH_CHECK();
    int64_t g = ceil_div(padded * b.Kp, 256);
    if (g > 152 * 16) g = 152 * 16;
    tc_build_kernel<<<static_cast<unsigned>(g), 256, 0, s>>>(xc, norms, n, d, b.Kp, b.dr, b.split, perm, padded,
                                                             reinterpret_cast<const TcScale*>(b.scale),
                                                             static_cast<__half*>(b.xh), static_cast<__half*>(b.xb),
                                                             b.xr, b.cn, b.ix);
    CG_LAUNCH_CHECK();
    return b;
}

void tc_seed(const TcBuffers& b, int t0, int mt, int d, int k, uint64_t* seed_keys, unsigned long long* kth_shared,
             cudaStream_t s) {
    const size_t smem = sizeof(float) * (static_cast<size_t>(kCT) * (b.dr + 1) + kCT);
    set_max_dynamic_smem(reinterpret_cast<const void*>(tc_seed_kernel), 100 * 1024);
    tc_seed_kernel<<<mt, 256, smem, s>>>(b.xr, b.ix, t0, d, b.dr, k, seed_keys, kth_shared);
    CG_LAUNCH_CHECK();
}

void tc_sweep(const TcBuffers& b, int nt, int t0, int mt, int nsplit, int d, int k, const unsigned* maxn,
              unsigned long long* kth_shared, uint64_t* partial, uint64_t* lists, int* status, cudaStream_t s, int qs,
              const uint2* plist, const int* pcount) {
    const size_t smem = sizeof(TcSmem) + 1024;
    set_max_dynamic_smem(reinterpret_cast<const void*>(tc_sweep_kernel), static_cast<int>(smem));
    const CUtensorMap map = tc::make_kmajor_map(b.xh, static_cast<int64_t>(nt) * kCT, b.Kp, true);
    const CUtensorMap mapb = tc::make_kmajor_map(b.xb, static_cast<int64_t>(nt) * kCT, b.Kp, true);
    // row tiles in batches, so that the list workspace stays bounded
    const int ntb_max = kTcMaxCtasPerLaunch / nsplit > 0 ? kTcMaxCtasPerLaunch / nsplit : 1;
    for (int T0 = t0; T0 < t0 + mt; T0 += ntb_max) {
        const int ntb = t0 + mt - T0 < ntb_max ? t0 + mt - T0 : ntb_max;
        tc_sweep_kernel<<<ntb * nsplit, kTcThreads, smem, s>>>(map, mapb, b.xr, b.cn, b.ix,
                                                               reinterpret_cast<const TcScale*>(b.scale), nt, T0, ntb,
                                                               nsplit, d, b.dr, b.Kp, b.split, b.ksteps, k, maxn,
                                                               kth_shared, partial, lists, status, qs, plist, pcount);
        CG_LAUNCH_CHECK();
    }
}

}  // namespace culof_gb300
