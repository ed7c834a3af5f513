// The fused distance + filtered exact select for wider points (8 < d <= 128),
// FP32 on the CUDA cores.
//
// Same algorithm as the small-d sweep (fast.cu): rows of a 128-point tile
// against column tiles in Morton order, e = |b|^2 - 2 a.b evaluated once per
// pair and compared with the row's rigorous threshold tau, passing pairs
// rescored exactly (direct differences, the oracle's formula) into per-row
// lists. What changes with d is the data movement: a GEMM-style tiling.
//   * the CTA's 128 rows stay in shared memory as -2a, dimension-major;
//   * each column tile streams in chunks of 16 dimensions x 128 columns
//     (cp.async, double buffered), dimension-major as well;
//   * each thread accumulates an 8-row x 8-column block with packed
//     fma.rn.f32x2 (two rows per instruction), 32 per dimension;
//   * after the last chunk of a tile the block is filtered; candidates go to
//     the owning warp's queue (each warp owns 16 rows) and are rescored with
//     the column's coordinates read from the tile in global memory (L2).
#include "common.cuh"
#include "engine.cuh"
#include "fast.cuh"
#include "sweep_common.cuh"

namespace culof_gb300 {

namespace {

using namespace sweep;

constexpr int kChunk = 16;  // dimensions per streamed chunk

// Wide tile t: coords [dpw][kCT] (dimension-major, zero padded), norms[kCT],
// index[kCT].
__host__ __device__ inline int64_t wide_tile_floats(int dpw) { return static_cast<int64_t>(dpw) * kCT + 2 * kCT; }

__global__ void build_wide_tiles_kernel(const float* __restrict__ xc, const float* __restrict__ norms, int64_t n,
                                        int d, int dpw, const unsigned* __restrict__ perm, int64_t padded,
                                        float* __restrict__ tiles) {
    for (int64_t p = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; p < padded;
         p += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t t = p / kCT;
        const int c = static_cast<int>(p % kCT);
        float* tile = tiles + t * wide_tile_floats(dpw);
        const bool valid = p < n;
        const unsigned orig = valid ? perm[p] : kNoIndex;
        for (int f = 0; f < dpw; ++f)
            tile[static_cast<int64_t>(f) * kCT + c] = (valid && f < d) ? xc[static_cast<int64_t>(orig) * d + f] : 0.0f;
        tile[static_cast<int64_t>(dpw) * kCT + c] = valid ? norms[orig] : __int_as_float(0x7fc00000);
        reinterpret_cast<unsigned*>(tile)[static_cast<int64_t>(dpw) * kCT + kCT + c] = orig;
    }
}

// Per row of tile T: the exact k best keys over the tile's own columns and
// the row's starting shared k-th key (as the small-d seed kernel).
__global__ void __launch_bounds__(kThreads) wide_seed_kernel(const float* __restrict__ tiles, int t0, int d, int dpw,
                                                             int k, uint64_t* __restrict__ seed_keys,
                                                             unsigned long long* __restrict__ kth_shared) {
    extern __shared__ __align__(16) float stile[];  // [dpw][kCT] coords, then kCT index
    const int T = t0 + static_cast<int>(blockIdx.x);
    const float* src = tiles + static_cast<int64_t>(T) * wide_tile_floats(dpw);
    const int nfl = dpw * kCT;
    for (int i = threadIdx.x; i < nfl; i += kThreads) stile[i] = src[i];
    unsigned* idx = reinterpret_cast<unsigned*>(stile + nfl);
    for (int i = threadIdx.x; i < kCT; i += kThreads)
        idx[i] = reinterpret_cast<const unsigned*>(src)[nfl + kCT + i];
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = warp; r < kRT; r += kWarps) {
        const int64_t pos = static_cast<int64_t>(T) * kRT + r;
        const bool row_valid = idx[r] != kNoIndex;
        // the lane's four columns as four independent chains (each in the
        // oracle's order), the row's coordinate loaded once per dimension
        float s4[4] = {0.0f, 0.0f, 0.0f, 0.0f};
#pragma unroll 4
        for (int f = 0; f < d; ++f) {
            const float a = stile[f * kCT + r];
#pragma unroll
            for (int j = 0; j < 4; ++j) {
                const float t = __fsub_rn(a, stile[f * kCT + j * 32 + lane]);
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

template <int M>
struct WideHead {
    RowLists<M> L;
    float bn[2][kCT];
    unsigned bi[2][kCT];
    uint16_t queue[kWarps][kQueueCap];
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_one() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// Column c of a thread's block: c < 4 -> 4 tx + c, else 64 + 4 tx + (c - 4),
// so each 16-byte shared load of a warp is contiguous across lanes.
__device__ __forceinline__ int block_col(int tx, int c) { return (c < 4) ? 4 * tx + c : 64 + 4 * tx + (c - 4); }

template <int M>
__device__ bool wide_drain(WideHead<M>& H, const float* __restrict__ A, int qc, const float* __restrict__ gtile,
                           int hb, int d, int k, float nmax, int dp_bound) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    bool compacted = false;
    for (int base = 0; base < qc; base += 32) {
        const int i = base + lane;
        if (i < qc) {
            const unsigned e = H.queue[warp][i];
            const int r = static_cast<int>(e >> 8), c = static_cast<int>(e & 0xFF);
            float s = 0.0f;
            for (int f = 0; f < d; ++f) {
                const float a = -0.5f * A[f * kRT + r];
                const float t = __fsub_rn(a, __ldg(gtile + static_cast<int64_t>(f) * kCT + c));
                s = __fmaf_rn(t, t, s);
            }
            const uint64_t key = make_key(__float_as_uint(s), H.bi[hb][c]);
            if (key < H.L.kth[r]) {
                const int slot = atomicAdd(&H.L.cnt[r], 1);
                H.L.list[r][slot] = key;
            }
        }
        __syncwarp();
        compacted |= compact_full_rows<M>(H.L, k, nmax, dp_bound);
    }
    return compacted;
}

template <int M>
__global__ void __launch_bounds__(kThreads, 1)
wide_sweep_kernel(const float* __restrict__ tiles, int nt, int t0, int mt, int nsplit, int d, int dpw, int k,
                  const unsigned* __restrict__ max_norm_bits, unsigned long long* __restrict__ kth_shared,
                  uint64_t* __restrict__ partial) {
    extern __shared__ __align__(128) unsigned char smem_raw[];
    WideHead<M>& H = *reinterpret_cast<WideHead<M>*>(smem_raw);
    float* A = reinterpret_cast<float*>(smem_raw + ((sizeof(WideHead<M>) + 127) & ~size_t(127)));  // [dpw][kRT]
    float* B = A + dpw * kRT;                                                                        // [2][kChunk][kCT]
    const int T = t0 + static_cast<int>(blockIdx.x) % mt;
    const int split = static_cast<int>(blockIdx.x) / mt;
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const float nmax = __uint_as_float(*max_norm_bits);
    const int64_t tfl = wide_tile_floats(dpw);
    const float* own = tiles + static_cast<int64_t>(T) * tfl;
    const int per = (nt - 1 + nsplit - 1) / nsplit;
    const int q0 = 1 + split * per;
    const int q1 = min(nt, q0 + per);
    const int count = q1 > q0 ? q1 - q0 : 0;
    const int nchunks = dpw / kChunk;
    const int dp_bound = dpw;  // length of the FMA chain behind e

    // rows: -2a (dimension-major), norms, shared k-th keys, thresholds
    for (int i = tid; i < dpw * kRT; i += kThreads) A[i] = -2.0f * own[i];
    if (tid < kRT) {
        const int64_t pos = static_cast<int64_t>(T) * kRT + tid;
        const float nr = own[static_cast<int64_t>(dpw) * kCT + tid];
        const uint64_t kk = kth_shared[pos];
        H.L.kth[tid] = kk;
        H.L.row_norm[tid] = nr;
        H.L.tau[tid] = (reinterpret_cast<const unsigned*>(own)[static_cast<int64_t>(dpw) * kCT + kCT + tid] == kNoIndex)
                           ? __int_as_float(0xff800000)
                           : tau_from(kk, nr, nmax, dp_bound);
        H.L.cnt[tid] = 0;
        H.L.sorted[tid] = 0;
    }

    auto issue = [&](int g) {
        const int m = g / nchunks, kc = g % nchunks;
        const float* tb = tiles + static_cast<int64_t>(spiral_tile(T, q0 + m, nt)) * tfl;
        float* dst = B + (g & 1) * kChunk * kCT;
        const float* srcc = tb + static_cast<int64_t>(kc) * kChunk * kCT;
        for (int s = tid; s < kChunk * kCT / 4; s += kThreads) cp_async16(dst + 4 * s, srcc + 4 * s);
        if (kc == 0) {
            const float* hdr = tb + static_cast<int64_t>(dpw) * kCT;
            if (tid < kCT / 4) cp_async16(&H.bn[m & 1][4 * tid], hdr + 4 * tid);
            else if (tid < kCT / 2) cp_async16(&H.bi[m & 1][4 * (tid - kCT / 4)], hdr + kCT + 4 * (tid - kCT / 4));
        }
        cp_async_commit();
    };

    const int total = count * nchunks;
    if (total > 0) issue(0);
    __syncthreads();

    const int rh = lane >> 4, tx = lane & 15;
    const int r0 = warp * kRowsPerWarp + rh * 8;
    uint64_t acc[4][8];
    uint64_t tau2p[4];
    float tau_r[8];
    auto load_tau = [&]() {
#pragma unroll
        for (int i = 0; i < 8; ++i) tau_r[i] = H.L.tau[r0 + i];
#pragma unroll
        for (int ip = 0; ip < 4; ++ip) {
            const float t0 = isinf(tau_r[2 * ip]) ? tau_r[2 * ip] : nextafterf(tau_r[2 * ip], __int_as_float(0x7f800000));
            const float t1 =
                isinf(tau_r[2 * ip + 1]) ? tau_r[2 * ip + 1] : nextafterf(tau_r[2 * ip + 1], __int_as_float(0x7f800000));
            tau2p[ip] = static_cast<uint64_t>(__float_as_uint(t0)) | (static_cast<uint64_t>(__float_as_uint(t1)) << 32);
        }
    };
    load_tau();

    for (int g = 0; g < total; ++g) {
        if (g + 1 < total) {
            issue(g + 1);
            cp_async_wait_one();
        } else {
            cp_async_wait_all();
        }
        __syncthreads();
        const int m = g / nchunks, kc = g % nchunks;
        const int hb = m & 1;
        if (kc == 0) {
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                const uint64_t nb = dup2(H.bn[hb][block_col(tx, c)]);
#pragma unroll
                for (int ip = 0; ip < 4; ++ip) acc[ip][c] = nb;
            }
        }
        const float* Bc = B + (g & 1) * kChunk * kCT;
        const float* Ac = A + kc * kChunk * kRT;
#pragma unroll 4
        for (int f = 0; f < kChunk; ++f) {
            const ulonglong2 a01 = *reinterpret_cast<const ulonglong2*>(Ac + f * kRT + r0);
            const ulonglong2 a23 = *reinterpret_cast<const ulonglong2*>(Ac + f * kRT + r0 + 4);
            const float4 b0 = *reinterpret_cast<const float4*>(Bc + f * kCT + 4 * tx);
            const float4 b1 = *reinterpret_cast<const float4*>(Bc + f * kCT + 64 + 4 * tx);
            const uint64_t a2[4] = {a01.x, a01.y, a23.x, a23.y};
            const uint64_t bd[8] = {dup2(b0.x), dup2(b0.y), dup2(b0.z), dup2(b0.w),
                                    dup2(b1.x), dup2(b1.y), dup2(b1.z), dup2(b1.w)};
#pragma unroll
            for (int c = 0; c < 8; ++c)
#pragma unroll
                for (int ip = 0; ip < 4; ++ip) acc[ip][c] = fma2(a2[ip], bd[c], acc[ip][c]);
        }
        if (kc == nchunks - 1) {
            // filter the finished 8 x 8 block; queue and rescore candidates
            const float* gtile = tiles + static_cast<int64_t>(spiral_tile(T, q0 + m, nt)) * tfl;
            int qc = 0;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                unsigned signs = 0;
#pragma unroll
                for (int ip = 0; ip < 4; ++ip) {
                    uint64_t dlt;
                    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(dlt) : "l"(acc[ip][c]), "l"(tau2p[ip]));
                    signs |= static_cast<unsigned>(dlt) | static_cast<unsigned>(dlt >> 32);
                }
                if (__any_sync(0xffffffffu, static_cast<int>(signs) < 0)) {
                    unsigned pass = 0;
#pragma unroll
                    for (int ip = 0; ip < 4; ++ip) {
                        pass |= (lo_f(acc[ip][c]) <= tau_r[2 * ip] ? 1u : 0u) << (2 * ip);
                        pass |= (hi_f(acc[ip][c]) <= tau_r[2 * ip + 1] ? 1u : 0u) << (2 * ip + 1);
                    }
                    int tot;
                    int off = warp_prefix_offset(__popc(pass), tot);
                    const int col = block_col(tx, c);
                    while (pass) {
                        const int b = __ffs(pass) - 1;
                        pass &= pass - 1;
                        H.queue[warp][qc + off++] = static_cast<uint16_t>(((r0 + b) << 8) | col);
                    }
                    qc += tot;
                    __syncwarp();
                    if (qc >= 32) {
                        if (wide_drain<M>(H, A, qc, gtile, hb, d, k, nmax, dp_bound)) load_tau();
                        qc = 0;
                    }
                }
            }
            if (qc > 0 && wide_drain<M>(H, A, qc, gtile, hb, d, k, nmax, dp_bound)) load_tau();
        }
        __syncthreads();
    }
    // final: this split's sorted k best per row; share the k-th key
    for (int i = 0; i < kRowsPerWarp; ++i) {
        const int r = warp * kRowsPerWarp + i;
        compact_row<M>(H.L, r, k, nmax, dp_bound);
        const int64_t pos = static_cast<int64_t>(T) * kRT + r;
        const int c = H.L.cnt[r];
        uint64_t* out = partial + (static_cast<int64_t>(split) * nt * kRT + pos) * k;
        for (int e = lane; e < k; e += 32) out[e] = e < c ? H.L.list[r][e] : kKeyMax;
        if (lane == 0 && H.L.kth[r] != kKeyMax) atomicMin(&kth_shared[pos], static_cast<unsigned long long>(H.L.kth[r]));
    }
}

template <int M>
size_t wide_smem_bytes(int dpw) {
    return ((sizeof(WideHead<M>) + 127) & ~size_t(127)) + sizeof(float) * (static_cast<size_t>(dpw) * kRT + 2 * kChunk * kCT);
}

template <int M>
void launch_wide_sweep_m(const float* tiles, int nt, int t0, int mt, int nsplit, int d, int dpw, int k,
                         const unsigned* maxn, unsigned long long* kth_shared, uint64_t* partial, cudaStream_t s) {
    const size_t smem = wide_smem_bytes<M>(dpw);
    CG_CUDA(cudaFuncSetAttribute(wide_sweep_kernel<M>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(smem)));
    wide_sweep_kernel<M><<<mt * nsplit, kThreads, smem, s>>>(tiles, nt, t0, mt, nsplit, d, dpw, k, maxn, kth_shared,
                                                             partial);
    CG_LAUNCH_CHECK();
}

}  // namespace

int wide_dims_padded(int d) { return ((d + kChunk - 1) / kChunk) * kChunk; }
size_t wide_tiles_floats(int d, int nt) { return static_cast<size_t>(wide_tile_floats(wide_dims_padded(d))) * nt; }

void wide_build_tiles(const float* xc, const float* norms, int64_t n, int d, const unsigned* perm, int nt,
                      float* tiles, cudaStream_t s) {
    const int64_t padded = static_cast<int64_t>(nt) * kCT;
    int64_t g = ceil_div(padded, 256);
    if (g > 152 * 8) g = 152 * 8;
    build_wide_tiles_kernel<<<static_cast<unsigned>(g), 256, 0, s>>>(xc, norms, n, d, wide_dims_padded(d), perm,
                                                                      padded, tiles);
    CG_LAUNCH_CHECK();
}

void wide_seed(const float* tiles, int nt, int t0, int mt, int d, int k, uint64_t* seed_keys,
               unsigned long long* kth_shared, cudaStream_t s) {
    (void)nt;
    const int dpw = wide_dims_padded(d);
    const size_t smem = sizeof(float) * (static_cast<size_t>(dpw) * kCT + kCT);
    CG_CUDA(cudaFuncSetAttribute(wide_seed_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem)));
    wide_seed_kernel<<<mt, kThreads, smem, s>>>(tiles, t0, d, dpw, k, seed_keys, kth_shared);
    CG_LAUNCH_CHECK();
}

void wide_sweep(const float* tiles, int nt, int t0, int mt, int nsplit, int d, int k, const unsigned* maxn,
                unsigned long long* kth_shared, uint64_t* partial, cudaStream_t s) {
    const int dpw = wide_dims_padded(d);
    // list capacities as the small-d sweep's (k + 32 free slots at least;
    // with 128 keys the shared memory stays within 218 KB at d = 128)
    if (k > 48) launch_wide_sweep_m<128>(tiles, nt, t0, mt, nsplit, d, dpw, k, maxn, kth_shared, partial, s);
    else if (k > 24) launch_wide_sweep_m<96>(tiles, nt, t0, mt, nsplit, d, dpw, k, maxn, kth_shared, partial, s);
    else launch_wide_sweep_m<64>(tiles, nt, t0, mt, nsplit, d, dpw, k, maxn, kth_shared, partial, s);
}

}  // namespace culof_gb300
