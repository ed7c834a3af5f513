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
//   * passing pairs are queued per warp and rescored exactly from FP32
//     row-major coordinates (the oracle's direct-difference formula) into
//     per-row lists; compaction, the shared k-th key and the merge are those
//     of the FP32 sweeps.
//
// Exactness: tau (tc_tau below) bounds the filter value of every column whose
// exact FP32 distance can still enter the row's k best, covering the f16
// rounding of both operands (relative 2^-11, absolute 2^-14 in scaled units
// for values that fall below the f16 normal range or are flushed), the f32
// accumulation of the tensor core (taken as K * 2^-20 relative), the float32
// norms and the float32 evaluation of f. Data whose scale cannot be brought
// into the f16 range (|S| > 62, or non-finite values) disable the filter:
// every pair is then rescored exactly.
#include <cuda_fp16.h>

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
// index (kNoIndex for padding).
__global__ void tc_build_kernel(const float* __restrict__ xc, const float* __restrict__ norms, int64_t n, int d,
                                int Kp, int dr, const unsigned* __restrict__ perm, int64_t padded,
                                const TcScale* __restrict__ scale, __half* __restrict__ xh, float* __restrict__ xr,
                                float* __restrict__ cn, unsigned* __restrict__ ix) {
    const float sc = scale->sc;
    const int64_t total = padded * Kp;
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t p = e / Kp;
        const int f = static_cast<int>(e % Kp);
        const bool valid = p < n;
        const unsigned orig = valid ? perm[p] : kNoIndex;
        const float x = (valid && f < d) ? xc[static_cast<int64_t>(orig) * d + f] : 0.0f;
        xh[e] = __float2half_rn(x * sc);
        if (f < dr) xr[p * dr + f] = x;
        if (f == 0) {
            cn[p] = valid ? norms[orig] : __int_as_float(0x7f800000);
            ix[p] = orig;
        }
    }
}

// Per row of tile T: the exact k best keys over the tile's own columns and
// the row's starting shared k-th key (as the FP32 seed kernels).
__global__ void __launch_bounds__(256) tc_seed_kernel(const float* __restrict__ xr, const unsigned* __restrict__ ix,
                                                      int d, int dr, int k, uint64_t* __restrict__ seed_keys,
                                                      unsigned long long* __restrict__ kth_shared) {
    extern __shared__ float spts[];  // [kCT][dr + 1]
    const int T = blockIdx.x;
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
        uint64_t v[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int c = j * 32 + lane;
            uint64_t key = kKeyMax;
            if (row_valid && c != r && idx[c] != kNoIndex) {
                float s = 0.0f;
                for (int f = 0; f < d; ++f) {
                    const float t = __fsub_rn(spts[r * ld + f], spts[c * ld + f]);
                    s = __fmaf_rn(t, t, s);
                }
                key = make_key(__float_as_uint(s), idx[c]);
            }
            v[j] = key;
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

// Rigorous threshold of the f16 filter for a row with float32 norm na whose
// current k-th key is kth (see the file comment). With D the k-th distance,
// u = 2^-24, g the relative error of the float32 norms, A, B upper bounds of
// |a| and |b|, the f16 Gram value G of a column b with exact distance <= D
// satisfies
//   |b|^2 - 2 a.b <= Tm - |a|^2,  Tm = D / (1 - (K + 2) u)
//   |G - a.b| <= E = (2 uh + uh^2) A B + eta (1 + uh) sqrt(K) (A + B) + K eta^2
//                    + K ua ((1 + uh) A + sqrt(K) eta) ((1 + uh) B + sqrt(K) eta)
// so f = fl(Nb - 2 G) <= Tm - na / (1 + g) + g / (1 - g) Nmax + 2 E
//                        + u (Nmax + 2 (A B + E)),
// plus 8u of slack for evaluating this in double and rounding it up.
__device__ float tc_tau(uint64_t kth, float na, float nmax, int K, float eta_f) {
    if (kth == kKeyMax) return __int_as_float(0x7f800000);
    const double D = static_cast<double>(__uint_as_float(key_bits(kth)));
    const double u = 5.9604644775390625e-08;  // 2^-24
    const double uh = 4.8828125e-04;          // 2^-11
    const double ua = 9.5367431640625e-07;    // 2^-20
    const double g = (K + 1) * u / (1.0 - (K + 1) * u);
    const double a = static_cast<double>(na), m = static_cast<double>(nmax), eta = static_cast<double>(eta_f);
    const double Tm = D / (1.0 - (K + 2) * u);
    const double A = sqrt(a / (1.0 - g)), B = sqrt(m / (1.0 - g));
    const double sk = sqrt(static_cast<double>(K));
    const double E = (2.0 * uh + uh * uh) * A * B + eta * (1.0 + uh) * sk * (A + B) + K * eta * eta +
                     K * ua * ((1.0 + uh) * A + sk * eta) * ((1.0 + uh) * B + sk * eta);
    double t = Tm - a / (1.0 + g) + g / (1.0 - g) * m + 2.0 * E + u * (m + 2.0 * (A * B + E));
    t += 8.0 * u * (Tm + a + m + 2.0 * A * B) + 1e-30;
    return __double2float_ru(t);
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

template <int M>
struct TcSmem {
    uint8_t a[2][kBox];              // row tile operand (K boxes 0..1)
    uint8_t b[kTcStages][2][kBox];   // column tile operands
    RowLists<M> L;
    uint16_t queue[kEpiWarps][kTcQueue];
    uint64_t full[kTcStages], empty[kTcStages], tfull[2], tempty[2], afull, fin;
    uint32_t tmem_base;
    int abort;
};

template <int M>
__device__ void tc_abort(TcSmem<M>& sh, int* status) {
    *reinterpret_cast<volatile int*>(&sh.abort) = 1;
    atomicExch(status, 1);
}
template <int M>
__device__ __forceinline__ bool tc_aborted(TcSmem<M>& sh) {
    return *reinterpret_cast<volatile int*>(&sh.abort) != 0;
}

// Compact every row of this epilogue warp (32 rows from row0) whose list has
// less than 32 free slots. True if any was.
template <int M>
__device__ bool tc_compact_full_rows(RowLists<M>& L, int row0, int k, float nmax, int dp) {
    const int lane = threadIdx.x & 31;
    unsigned full = __ballot_sync(0xffffffffu, L.cnt[row0 + lane] > M - 32);
    const bool any = full != 0;
    while (full) {
        compact_row<M>(L, row0 + __ffs(full) - 1, k, nmax, dp);
        full &= full - 1;
    }
    return any;
}

// Rescore the warp's queued pairs of column tile `tile` exactly and add the
// keys that beat their row's k-th key. True if a list was compacted.
template <int M>
__device__ bool tc_drain(TcSmem<M>& sh, int wq, int row0, int qc, int64_t rbase, int64_t cbase,
                         const float* __restrict__ xr, const unsigned* __restrict__ ix, int d, int dr, int k,
                         float nmax, int Kp) {
    const int lane = threadIdx.x & 31;
    bool compacted = false;
    for (int base = 0; base < qc; base += 32) {
        const int i = base + lane;
        if (i < qc) {
            const unsigned e = sh.queue[wq][i];
            const int r = static_cast<int>(e >> 8), c = static_cast<int>(e & 0xFF);
            const unsigned ib = __ldg(ix + cbase + c);
            if (ib != kNoIndex) {
                const float4* pa = reinterpret_cast<const float4*>(xr + (rbase + r) * dr);
                const float4* pb = reinterpret_cast<const float4*>(xr + (cbase + c) * dr);
                float s = 0.0f;
                for (int f4 = 0; 4 * f4 < d; ++f4) {
                    const float4 x = __ldg(pa + f4), y = __ldg(pb + f4);
                    const float xa[4] = {x.x, x.y, x.z, x.w}, yb[4] = {y.x, y.y, y.z, y.w};
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        if (4 * f4 + q < d) {
                            const float t = __fsub_rn(xa[q], yb[q]);
                            s = __fmaf_rn(t, t, s);
                        }
                    }
                }
                const uint64_t key = make_key(__float_as_uint(s), ib);
                if (key < sh.L.kth[r]) {
                    const int slot = atomicAdd(&sh.L.cnt[r], 1);
                    sh.L.list[r][slot] = key;
                }
            }
        }
        __syncwarp();
        compacted |= tc_compact_full_rows<M>(sh.L, row0, k, nmax, Kp);
    }
    return compacted;
}

template <int M>
__global__ void __launch_bounds__(kTcThreads, 1)
tc_sweep_kernel(const __grid_constant__ CUtensorMap tmap, const float* __restrict__ xr,
                const float* __restrict__ cn, const unsigned* __restrict__ ix, const TcScale* __restrict__ scale,
                int nt, int nsplit, int d, int dr, int Kp, int k, const unsigned* __restrict__ max_norm_bits,
                unsigned long long* __restrict__ kth_shared, uint64_t* __restrict__ partial, int* __restrict__ status) {
    extern __shared__ uint8_t tc_raw[];
    TcSmem<M>& sh = *reinterpret_cast<TcSmem<M>*>((reinterpret_cast<uintptr_t>(tc_raw) + 1023) & ~uintptr_t(1023));
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int T = blockIdx.x % nt;
    const int split = blockIdx.x / nt;
    const int per = (nt - 1 + nsplit - 1) / nsplit;
    const int q0 = 1 + split * per;
    const int q1 = min(nt, q0 + per);
    const int count = q1 > q0 ? q1 - q0 : 0;
    const int nkb = Kp / 64;
    const float nmax = __uint_as_float(*max_norm_bits);
    const int64_t rbase = static_cast<int64_t>(T) * kRT;

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
        sh.L.kth[r] = kth_shared[rbase + r];
        sh.L.row_norm[r] = cn[rbase + r];
        sh.L.tau[r] = 0.0f;
        sh.L.cnt[r] = 0;
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
                const int col0 = spiral_tile(T, q0 + j, nt) * kCT;
                mbar_expect_tx(&sh.full[s], nkb * kBox);
                for (int kb = 0; kb < nkb; ++kb) tc::tma_load_2d(sh.b[s][kb], &tmap, 64 * kb, col0, &sh.full[s]);
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
                for (int kk = 0; kk < 4 * nkb; ++kk) {
                    const int kb = kk >> 2, sub = kk & 3;
                    const uint64_t ad = tc::sw128_desc(smem_u32(sh.a[kb]) + 32 * sub);
                    const uint64_t bd = tc::sw128_desc(smem_u32(sh.b[s][kb]) + 32 * sub);
                    tc::mma_bf16(dt, ad, bd, idesc, kk > 0);
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
        const TcScale sc = *scale;
        const bool all = sc.all != 0.0f;
        const bool row_valid = __ldg(ix + rbase + r) != kNoIndex;
        const float na = sh.L.row_norm[r];
        auto row_tau = [&]() -> float {
            return row_valid ? tc_tau(sh.L.kth[r], na, nmax, Kp, sc.eta) : __int_as_float(0xff800000);
        };
        uint64_t tq = tau_pair(row_tau());
        const uint64_t k2 = dup2(sc.k2);
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(row0) << 16);
        for (int j = 0; j < count; ++j) {
            const int acc = j & 1;
            if (!mbar_wait_warp(&sh.tfull[acc], (j >> 1) & 1)) {
                if (lane == 0) tc_abort(sh, status);
                break;
            }
            tc::tc_fence_after();
            const int64_t cbase = static_cast<int64_t>(spiral_tile(T, q0 + j, nt)) * kCT;
            const float4* cn4 = reinterpret_cast<const float4*>(cn + cbase);
            int qc = 0;
#pragma unroll 1
            for (int ch = 0; ch < 4; ++ch) {
                float g[32];
                tc::tmem_ld32(lane_addr + static_cast<uint32_t>(acc * 128 + 32 * ch), g);
                uint64_t dl[16];
                unsigned signs = 0;
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    const float4 nb = __ldg(cn4 + 8 * ch + q);
                    const uint64_t f0 = fma2(pack2(g[4 * q], g[4 * q + 1]), k2, pack2(nb.x, nb.y));
                    const uint64_t f1 = fma2(pack2(g[4 * q + 2], g[4 * q + 3]), k2, pack2(nb.z, nb.w));
                    dl[2 * q] = sub2(f0, tq);
                    dl[2 * q + 1] = sub2(f1, tq);
                    signs |= static_cast<unsigned>(dl[2 * q]) | static_cast<unsigned>(dl[2 * q] >> 32) |
                             static_cast<unsigned>(dl[2 * q + 1]) | static_cast<unsigned>(dl[2 * q + 1] >> 32);
                }
                if (all) signs = row_valid ? 0x80000000u : 0u;
                if (__any_sync(0xffffffffu, static_cast<int>(signs) < 0)) {
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
                    int tot;
                    int off = warp_prefix_offset(__popc(pass), tot);
                    while (pass) {
                        const int b = __ffs(pass) - 1;
                        pass &= pass - 1;
                        sh.queue[wq][qc + off++] = static_cast<uint16_t>((r << 8) | (32 * ch + b));
                    }
                    qc += tot;
                    __syncwarp();
                    if (qc >= 32) {
                        if (tc_drain<M>(sh, wq, row0, qc, rbase, cbase, xr, ix, d, dr, k, nmax, Kp))
                            tq = tau_pair(row_tau());
                        qc = 0;
                    }
                }
            }
            // the accumulator is free for the next tile but one
            tc::tc_fence_before();
            __syncwarp();
            if (lane == 0) mbar_arrive(&sh.tempty[acc]);
            if (qc > 0 && tc_drain<M>(sh, wq, row0, qc, rbase, cbase, xr, ix, d, dr, k, nmax, Kp))
                tq = tau_pair(row_tau());
        }
        // this split's sorted k best per row; share the k-th key
        for (int i = 0; i < 32; ++i) {
            const int rr = row0 + i;
            compact_row<M>(sh.L, rr, k, nmax, Kp);
            const int64_t pos = rbase + rr;
            const int c = sh.L.cnt[rr];
            uint64_t* out = partial + (static_cast<int64_t>(split) * nt * kRT + pos) * k;
            for (int e = lane; e < k; e += 32) out[e] = e < c ? sh.L.list[rr][e] : kKeyMax;
            if (lane == 0 && sh.L.kth[rr] != kKeyMax)
                atomicMin(&kth_shared[pos], static_cast<unsigned long long>(sh.L.kth[rr]));
        }
    }
    tc::tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc::tc_fence_after();
        tc::tmem_dealloc(tmem, kTmemCols);
    }
}

template <int M>
void launch_tc_sweep_m(const TcBuffers& b, int nt, int nsplit, int d, int k, const unsigned* maxn,
                       unsigned long long* kth_shared, uint64_t* partial, int* status, cudaStream_t s) {
    const size_t smem = sizeof(TcSmem<M>) + 1024;
    static bool configured = false;
    if (!configured) {
        CG_CUDA(cudaFuncSetAttribute(tc_sweep_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
        configured = true;
    }
    const CUtensorMap map = tc::make_kmajor_map(b.xh, static_cast<int64_t>(nt) * kCT, b.Kp, true);
    tc_sweep_kernel<M><<<nt * nsplit, kTcThreads, smem, s>>>(map, b.xr, b.cn, b.ix,
                                                            reinterpret_cast<const TcScale*>(b.scale), nt, nsplit, d,
                                                            b.dr, b.Kp, k, maxn, kth_shared, partial, status);
    CG_LAUNCH_CHECK();
}

}  // namespace

size_t tc_buffer_bytes(int64_t padded, int d) {
    const int Kp = d <= 64 ? 64 : 128;
    const int dr = (d + 3) & ~3;
    const auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    return up(sizeof(__half) * padded * Kp) + up(sizeof(float) * padded * dr) + up(sizeof(float) * padded) +
           up(sizeof(unsigned) * padded) + up(sizeof(TcScale));
}

TcBuffers tc_prepare(void* buf, const float* xc, const float* norms, int64_t n, int d, const unsigned* perm, int nt,
                     const unsigned* minmax, cudaStream_t s) {
    const int64_t padded = static_cast<int64_t>(nt) * kCT;
    const auto up = [](size_t x) { return (x + 255) & ~static_cast<size_t>(255); };
    TcBuffers b;
    b.Kp = d <= 64 ? 64 : 128;
    b.dr = (d + 3) & ~3;
    char* p = static_cast<char*>(buf);
    b.xh = p;
    p += up(sizeof(__half) * padded * b.Kp);
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
    tc_build_kernel<<<static_cast<unsigned>(g), 256, 0, s>>>(xc, norms, n, d, b.Kp, b.dr, perm, padded,
                                                             reinterpret_cast<const TcScale*>(b.scale),
                                                             static_cast<__half*>(b.xh), b.xr, b.cn, b.ix);
    CG_LAUNCH_CHECK();
    return b;
}

void tc_seed(const TcBuffers& b, int nt, int d, int k, uint64_t* seed_keys, unsigned long long* kth_shared,
             cudaStream_t s) {
    const size_t smem = sizeof(float) * (static_cast<size_t>(kCT) * (b.dr + 1) + kCT);
    static bool configured = false;
    if (!configured) {
        CG_CUDA(cudaFuncSetAttribute(tc_seed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, 100 * 1024));
        configured = true;
    }
    tc_seed_kernel<<<nt, 256, smem, s>>>(b.xr, b.ix, d, b.dr, k, seed_keys, kth_shared);
    CG_LAUNCH_CHECK();
}

void tc_sweep(const TcBuffers& b, int nt, int nsplit, int d, int k, const unsigned* maxn,
              unsigned long long* kth_shared, uint64_t* partial, int* status, cudaStream_t s) {
    if (k > 32) launch_tc_sweep_m<96>(b, nt, nsplit, d, k, maxn, kth_shared, partial, status, s);
    else launch_tc_sweep_m<64>(b, nt, nsplit, d, k, maxn, kth_shared, partial, status, s);
}

}  // namespace culof_gb300
