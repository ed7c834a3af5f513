// Sparse backward of the LOF scores with respect to the points (no reference
// counterpart: the reference computes scores only).
//
// With the neighbour sets N(i) held fixed (the k slots of a forward k-NN
// result, slot k-1 designating a k-th neighbour), the forward chain is
//   d2_ij   = |xc_i - xc_j|^2                         j in N(i)
//   kd2_j   = d2_{j, slot k-1}                         (squared k-distance)
//   reach_ij = sqrt(max(kd2_j, d2_ij))
//   lrd_i   = 1 / (sum_j reach_ij / k + 1e-10)         (lof.cu:32-46 of the reference)
//   score_i = sum_j lrd_j / (k lrd_i)                   (lof.cu:49-62)
// and xc = (x - mean) (* inv_std when normalising, population std, scale 1
// for zero-variance features). Given g = dL/dscore, the backward is evaluated
// in FP64 and is bit-reproducible: every sum over a point's reverse
// neighbours (the pairs (i, t) whose slot t names it) runs in a fixed order,
// taken from a stable radix sort of the slots by neighbour index (a
// transposed k-NN list), so no floating-point atomics are used.
//
// Subgradient conventions: max(kd2_j, d2_ij) sends the gradient to d2_ij when
// d2_ij > kd2_j and to kd2_j otherwise (ties go to the k-distance); a zero
// reach distance contributes no gradient (sqrt is not differentiable at 0).
#include "common.cuh"
#include "engine.cuh"
#include "fast.cuh"
#include "prep.cuh"

namespace culof_gb300 {

namespace {

__device__ __forceinline__ void flag_bad(int* status) { atomicExch(status, 2); }
// Indices used for addressing are clamped into [0, n): an invalid neighbour
// index (reported through the status word by bw_pair_kernel) gives a wrong
// gradient, never an out-of-range access.
__device__ __forceinline__ int64_t clampj(int32_t j, int64_t n) { return j < 0 ? 0 : (j >= n ? n - 1 : j); }

// The per-point sums below run one warp per point: lanes take the terms
// lane, lane + 32, ... in order and a fixed xor-shuffle tree adds the lanes'
// partials, so every sum has one fixed order and the gradient is
// bit-reproducible.
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = __dadd_rn(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}
__device__ __forceinline__ int64_t warp_id() { return (static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5; }
__device__ __forceinline__ int64_t warp_count() { return (static_cast<int64_t>(gridDim.x) * blockDim.x) >> 5; }

// d2[e] (e = t * n + i, the layout of the k-NN slots) in FP64 from the raw
// points: (x_i - x_j) * inv_std, the mean cancels. A warp per point, lanes
// over dimensions.
__global__ void bw_pair_kernel(const float* __restrict__ x, int64_t n, int d, int k, const int32_t* __restrict__ nbr,
                               const double* __restrict__ inv, double* __restrict__ d2, int* __restrict__ status) {
    const int lane = threadIdx.x & 31;
    for (int64_t i = warp_id(); i < n; i += warp_count()) {
        const float* xi = x + i * d;
        for (int t = 0; t < k; ++t) {
            const int64_t e = static_cast<int64_t>(t) * n + i;
            const int32_t j = nbr[e];
            double s = 0.0;
            if (j < 0 || j >= n) {
                if (lane == 0) flag_bad(status);
            } else {
                const float* xj = x + static_cast<int64_t>(j) * d;
                for (int f = lane; f < d; f += 32) {
                    const double u = __dmul_rn(__dsub_rn(static_cast<double>(xi[f]), static_cast<double>(xj[f])), inv[f]);
                    s = __fma_rn(u, u, s);
                }
            }
            s = warp_sum(s);
            if (lane == 0) d2[e] = s;
        }
    }
}

// Per point: reach distances of its slots, lrd. A warp per point, lanes over slots.
__global__ void bw_lrd_kernel(int64_t n, int k, const int32_t* __restrict__ nbr, const double* __restrict__ d2,
                              double* __restrict__ reach, double* __restrict__ lrd) {
    const int lane = threadIdx.x & 31;
    for (int64_t i = warp_id(); i < n; i += warp_count()) {
        double R = 0.0;
        for (int t = lane; t < k; t += 32) {
            const int64_t e = static_cast<int64_t>(t) * n + i;
            const int64_t j = clampj(nbr[e], n);
            const double kd = d2[static_cast<int64_t>(k - 1) * n + j];
            const double r = __dsqrt_rn(fmax(kd, d2[e]));
            reach[e] = r;
            R = __dadd_rn(R, r);
        }
        R = warp_sum(R);
        if (lane == 0) lrd[i] = __ddiv_rn(1.0, __dadd_rn(__ddiv_rn(R, static_cast<double>(k)), 1e-10));
    }
}

// Per point: S_i = sum_j lrd_j and the score. A warp per point.
__global__ void bw_score_kernel(int64_t n, int k, const int32_t* __restrict__ nbr, const double* __restrict__ lrd,
                                double* __restrict__ S, double* __restrict__ score) {
    const int lane = threadIdx.x & 31;
    for (int64_t i = warp_id(); i < n; i += warp_count()) {
        double s = 0.0;
        for (int t = lane; t < k; t += 32) s = __dadd_rn(s, lrd[clampj(nbr[static_cast<int64_t>(t) * n + i], n)]);
        s = warp_sum(s);
        if (lane == 0) {
            S[i] = s;
            if (score) score[i] = __ddiv_rn(s, __dmul_rn(static_cast<double>(k), lrd[i]));
        }
    }
}

// Transposed slot list: count slots per neighbour index (integer atomics,
// order-free), keys/values for the stable sort.
__global__ void bw_rev_init_kernel(int64_t n, int64_t total, const int32_t* __restrict__ nbr, unsigned* __restrict__ keys,
                                   unsigned* __restrict__ vals, unsigned* __restrict__ counts) {
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const unsigned j = static_cast<unsigned>(clampj(nbr[e], n));
        keys[e] = j;
        vals[e] = static_cast<unsigned>(e);
        atomicAdd(&counts[j], 1u);
    }
}

// dL/dlrd_m = -g_m S_m / (k lrd_m^2) + sum over reverse slots (i, t) of g_i / (k lrd_i).
// (A warp per point, lanes over the reverse slots.)
__global__ void bw_glrd_kernel(int64_t n, int k, const double* __restrict__ g, const double* __restrict__ lrd,
                               const double* __restrict__ S, const unsigned* __restrict__ off,
                               const unsigned* __restrict__ rev, double* __restrict__ glrd) {
    const double dk = static_cast<double>(k);
    const int lane = threadIdx.x & 31;
    for (int64_t m = warp_id(); m < n; m += warp_count()) {
        double acc = 0.0;
        for (unsigned p = off[m] + lane; p < off[m + 1]; p += 32) {
            const int64_t i = static_cast<int64_t>(rev[p]) % n;
            acc = __dadd_rn(acc, __ddiv_rn(g[i], __dmul_rn(dk, lrd[i])));
        }
        acc = warp_sum(acc);
        if (lane == 0) {
            const double lm = lrd[m];
            glrd[m] = __dadd_rn(-__ddiv_rn(__dmul_rn(g[m], S[m]), __dmul_rn(dk, __dmul_rn(lm, lm))), acc);
        }
    }
}

// Per slot: the reach-distance gradient c = dL/dR_i / (2 reach), routed to
// d2_ij (gd2) or to kd2_j (gkd).
__global__ void bw_route_kernel(int64_t n, int k, const int32_t* __restrict__ nbr, const double* __restrict__ d2,
                                const double* __restrict__ reach, const double* __restrict__ lrd,
                                const double* __restrict__ glrd, double* __restrict__ gd2, double* __restrict__ gkd) {
    const int64_t total = n * k;
    const double dk = static_cast<double>(k);
    for (int64_t e = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; e < total;
         e += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int64_t i = e % n;
        const int64_t j = clampj(nbr[e], n);
        const double li = lrd[i];
        const double gR = -__ddiv_rn(__dmul_rn(glrd[i], __dmul_rn(li, li)), dk);
        const double r = reach[e];
        const double c = r > 0.0 ? __ddiv_rn(gR, __dmul_rn(2.0, r)) : 0.0;
        const double kd = d2[static_cast<int64_t>(k - 1) * n + j];
        const bool via_d2 = d2[e] > kd;
        gd2[e] = via_d2 ? c : 0.0;
        gkd[e] = via_d2 ? 0.0 : c;
    }
}

// Per point j: the k-distance gradient (sum over its reverse slots, fixed
// order) joins the gradient of its own slot k-1.
// (A warp per point.)
__global__ void bw_kd_kernel(int64_t n, int k, const unsigned* __restrict__ off, const unsigned* __restrict__ rev,
                             const double* __restrict__ gkd, double* __restrict__ gd2) {
    const int lane = threadIdx.x & 31;
    for (int64_t j = warp_id(); j < n; j += warp_count()) {
        double s = 0.0;
        for (unsigned p = off[j] + lane; p < off[j + 1]; p += 32) s = __dadd_rn(s, gkd[rev[p]]);
        s = warp_sum(s);
        if (lane == 0) {
            const int64_t e = static_cast<int64_t>(k - 1) * n + j;
            gd2[e] = __dadd_rn(gd2[e], s);
        }
    }
}

// Gradient with respect to the normalised coordinates, one warp per point
// (lanes over dimensions): sum_t 2 gd2 (xc_i - xc_j) over its own slots minus
// the same over its reverse slots.
__global__ void bw_gx_kernel(const float* __restrict__ x, int64_t n, int d, int k, const int32_t* __restrict__ nbr,
                             const double* __restrict__ inv, const double* __restrict__ gd2,
                             const unsigned* __restrict__ off, const unsigned* __restrict__ rev,
                             double* __restrict__ gxc) {
    const int lane = threadIdx.x & 31;
    const int64_t warps = static_cast<int64_t>(gridDim.x) * (blockDim.x >> 5);
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * (blockDim.x >> 5) + (threadIdx.x >> 5); i < n; i += warps) {
        const float* xi = x + i * d;
        for (int f0 = 0; f0 < d; f0 += 32) {
            const int f = f0 + lane;
            const bool on = f < d;
            const double xif = on ? static_cast<double>(xi[f]) : 0.0;
            const double iv = on ? inv[f] : 0.0;
            double acc = 0.0;
            for (int t = 0; t < k; ++t) {
                const int64_t e = static_cast<int64_t>(t) * n + i;
                const double g2 = __dmul_rn(2.0, gd2[e]);
                if (on) {
                    const double diff = __dmul_rn(__dsub_rn(xif, static_cast<double>(x[clampj(nbr[e], n) * d + f])), iv);
                    acc = __fma_rn(g2, diff, acc);
                }
            }
            for (unsigned p = off[i]; p < off[i + 1]; ++p) {
                const unsigned e = rev[p];
                const int64_t m = static_cast<int64_t>(e) % n;
                const double g2 = __dmul_rn(2.0, gd2[e]);
                if (on) {
                    const double diff = __dmul_rn(__dsub_rn(static_cast<double>(x[m * d + f]), xif), iv);
                    acc = __fma_rn(-g2, diff, acc);
                }
            }
            if (on) gxc[i * d + f] = acc;
        }
    }
}

// Per (chunk of kCenterChunk rows, feature): partial sums of gxc and of
// gxc * xc; then per feature over the chunks. One block per chunk: warp w
// sums rows w, w + 8, ... of the chunk in order (lanes over features), and
// the 8 warps' partials are added in warp order.
constexpr int kColMaxD = 128;
__global__ void __launch_bounds__(256) bw_col_partials_kernel(const float* __restrict__ x, int64_t n, int d,
                                                              const double* __restrict__ mean,
                                                              const double* __restrict__ inv,
                                                              const double* __restrict__ gxc,
                                                              double* __restrict__ pa, double* __restrict__ pb) {
    __shared__ double sa[8][kColMaxD], sb[8][kColMaxD];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int64_t chunks = ceil_div(n, kCenterChunk);
    for (int64_t c = blockIdx.x; c < chunks; c += gridDim.x) {
        const int64_t r1 = (c + 1) * kCenterChunk < n ? (c + 1) * kCenterChunk : n;
        for (int fb = 0; fb < d; fb += kColMaxD) {  // blocks of features that fit the shared arrays
            const int fe = d - fb < kColMaxD ? d - fb : kColMaxD;
            for (int f0 = 0; f0 < fe; f0 += 32) {
                const int fl = f0 + lane, f = fb + fl;
                if (fl < fe) {
                    double a = 0.0, b = 0.0;
                    const double mf = mean[f], vf = inv[f];
                    for (int64_t r = c * kCenterChunk + warp; r < r1; r += 8) {
                        const double g = gxc[r * d + f];
                        const double xc = __dmul_rn(__dsub_rn(static_cast<double>(x[r * d + f]), mf), vf);
                        a = __dadd_rn(a, g);
                        b = __fma_rn(g, xc, b);
                    }
                    sa[warp][fl] = a;
                    sb[warp][fl] = b;
                }
            }
            __syncthreads();
            for (int fl = threadIdx.x; fl < fe; fl += blockDim.x) {
                double a = 0.0, b = 0.0;
                for (int w = 0; w < 8; ++w) {
                    a = __dadd_rn(a, sa[w][fl]);
                    b = __dadd_rn(b, sb[w][fl]);
                }
                pa[c * d + fb + fl] = a;
                pb[c * d + fb + fl] = b;
            }
            __syncthreads();
        }
    }
}

// Per feature: column means A_f = mean(gxc), B_f = mean(gxc * xc) and whether
// the feature was scaled (normalising and std > 1e-12, the rule of the
// forward centring).
// (A warp per feature, lanes over the chunks; the variance partials are
// summed in chunk order, as the forward centring sums them.)
__global__ void bw_col_finalize_kernel(int64_t n, int d, int normalize, const double* __restrict__ pa,
                                       const double* __restrict__ pb, const double* __restrict__ var_partial,
                                       double* __restrict__ A, double* __restrict__ B, int* __restrict__ scaled) {
    const int lane = threadIdx.x & 31;
    const int64_t chunks = ceil_div(n, kCenterChunk);
    const double dn = static_cast<double>(n);
    for (int64_t f = warp_id(); f < d; f += warp_count()) {
        double a = 0.0, b = 0.0;
        for (int64_t c = lane; c < chunks; c += 32) {
            a = __dadd_rn(a, pa[c * d + f]);
            b = __dadd_rn(b, pb[c * d + f]);
        }
        a = warp_sum(a);
        b = warp_sum(b);
        if (lane == 0) {
            double v = 0.0;
            if (normalize)
                for (int64_t c = 0; c < chunks; ++c) v = __dadd_rn(v, var_partial[c * d + f]);
            A[f] = __ddiv_rn(a, dn);
            B[f] = __ddiv_rn(b, dn);
            scaled[f] = normalize && __dsqrt_rn(__ddiv_rn(v, dn)) > 1e-12;
        }
    }
}

// dL/dx: centring (and scaling) backward of the normalised-coordinate gradient.
__global__ void bw_apply_kernel(const float* __restrict__ x, int64_t n, int d, const double* __restrict__ mean,
                                const double* __restrict__ inv, const double* __restrict__ gxc,
                                const double* __restrict__ A, const double* __restrict__ B,
                                const int* __restrict__ scaled, double* __restrict__ gx) {
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < n * d;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int f = static_cast<int>(t % d);
        const double g = __dsub_rn(gxc[t], A[f]);
        if (scaled[f]) {
            const double xc = __dmul_rn(__dsub_rn(static_cast<double>(x[t]), mean[f]), inv[f]);
            gx[t] = __dmul_rn(inv[f], __fma_rn(-xc, B[f], g));
        } else {
            gx[t] = g;
        }
    }
}

int grid_of(int64_t items) {
    int64_t g = ceil_div(items, 256);
    if (g > 152 * 16) g = 152 * 16;
    return static_cast<int>(g < 1 ? 1 : g);
}

}  // namespace

void Engine::lof_backward_device(const float* d_x, int64_t n, int d, int k, bool normalize, const int32_t* nbr_idx,
                                 const double* grad_scores, double* grad_x, double* scores_out) {
    validate_lof_args(d_x, n, d, k);
    if (!nbr_idx || !grad_scores || !grad_x) throw Error(kInvalidArgument, "device pointers must not be null");
    if (n * static_cast<int64_t>(k) > 0x7FFFFFFFll)
        throw Error(kInvalidArgument, "the backward takes n_points * k < 2^31 neighbour slots");
    CG_CUDA(cudaSetDevice(device_));
    cudaStream_t s = stream_;
    const int64_t total = n * k;
    const size_t nk = static_cast<size_t>(total);
    // statistics of the forward centring (same kernels, same order)
    float* xc = xc_.as<float>(static_cast<size_t>(n) * d);
    double* partial = partial_.as<double>(center_partial_count(n, d));
    double* mean = mean_.as<double>(d);
    double* inv = inv_std_.as<double>(d);
    CG_CUDA(cudaMemsetAsync(status_ptr(), 0, sizeof(int), s));
    center(d_x, n, d, normalize, xc, partial, mean, inv, s);

    // workspace: FP64 slot arrays, per-point arrays, the transposed slot list
    const size_t chunks_d = center_partial_count(n, d);
    char* w = static_cast<char*>(bw_.get(sizeof(double) * (4 * nk + 4 * static_cast<size_t>(n) +
                                                          2 * chunks_d + 2 * static_cast<size_t>(d) +
                                                          static_cast<size_t>(n) * d) +
                                         sizeof(unsigned) * (4 * nk + static_cast<size_t>(n) + 1 +
                                                             sort_pairs_counts(total)) +
                                         sizeof(int) * static_cast<size_t>(d) + 32 * 256));
    auto take = [&](size_t bytes) {
        char* p = w;
        w += (bytes + 255) & ~static_cast<size_t>(255);
        return p;
    };
    double* d2 = reinterpret_cast<double*>(take(sizeof(double) * nk));
    double* reach = reinterpret_cast<double*>(take(sizeof(double) * nk));
    double* gd2 = reinterpret_cast<double*>(take(sizeof(double) * nk));
    double* gkd = reinterpret_cast<double*>(take(sizeof(double) * nk));
    double* lrd = reinterpret_cast<double*>(take(sizeof(double) * n));
    double* S = reinterpret_cast<double*>(take(sizeof(double) * n));
    double* glrd = reinterpret_cast<double*>(take(sizeof(double) * n));
    double* gxc = reinterpret_cast<double*>(take(sizeof(double) * n * d));
    double* pa = reinterpret_cast<double*>(take(sizeof(double) * chunks_d));
    double* pb = reinterpret_cast<double*>(take(sizeof(double) * chunks_d));
    double* A = reinterpret_cast<double*>(take(sizeof(double) * d));
    double* B = reinterpret_cast<double*>(take(sizeof(double) * d));
    int* scaled = reinterpret_cast<int*>(take(sizeof(int) * d));
    unsigned* keys = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * nk));
    unsigned* vals = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * nk));
    unsigned* keys2 = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * nk));
    unsigned* vals2 = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * nk));
    unsigned* off = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * (n + 1)));
    unsigned* counts = reinterpret_cast<unsigned*>(take(sizeof(unsigned) * sort_pairs_counts(total)));
    int* status = status_ptr();
    double* score = scores_out;

    bw_pair_kernel<<<grid_of(n * 32), 256, 0, s>>>(d_x, n, d, k, nbr_idx, inv, d2, status);
    CG_LAUNCH_CHECK();
    bw_lrd_kernel<<<grid_of(n * 32), 256, 0, s>>>(n, k, nbr_idx, d2, reach, lrd);
    CG_LAUNCH_CHECK();
    bw_score_kernel<<<grid_of(n * 32), 256, 0, s>>>(n, k, nbr_idx, lrd, S, score);
    CG_LAUNCH_CHECK();
    // transposed slots: offsets from the per-index counts, slots in (t, i)
    // enumeration order within each index (stable sort)
    CG_CUDA(cudaMemsetAsync(off, 0, sizeof(unsigned) * (n + 1), s));
    bw_rev_init_kernel<<<grid_of(total), 256, 0, s>>>(n, total, nbr_idx, keys, vals, off);
    CG_LAUNCH_CHECK();
    exclusive_scan_u32(off, n + 1, s);
    int bits = 8;
    while (bits < 32 && (static_cast<int64_t>(1) << bits) < n) bits += 8;
    unsigned* rev = nullptr;
    sort_pairs_stable(keys, vals, keys2, vals2, total, bits, counts, s, &rev);

    bw_glrd_kernel<<<grid_of(n * 32), 256, 0, s>>>(n, k, grad_scores, lrd, S, off, rev, glrd);
    CG_LAUNCH_CHECK();
    bw_route_kernel<<<grid_of(total), 256, 0, s>>>(n, k, nbr_idx, d2, reach, lrd, glrd, gd2, gkd);
    CG_LAUNCH_CHECK();
    bw_kd_kernel<<<grid_of(n * 32), 256, 0, s>>>(n, k, off, rev, gkd, gd2);
    CG_LAUNCH_CHECK();
    bw_gx_kernel<<<grid_of(n * 32), 256, 0, s>>>(d_x, n, d, k, nbr_idx, inv, gd2, off, rev, gxc);
    CG_LAUNCH_CHECK();
    // the centring statistics' partials of (x - mean)^2 are still in `partial`
    // when normalising (the second pass of center())
    const int64_t col_chunks = ceil_div(n, kCenterChunk);
    bw_col_partials_kernel<<<static_cast<int>(col_chunks < 152 * 8 ? col_chunks : 152 * 8), 256, 0, s>>>(
        d_x, n, d, mean, inv, gxc, pa, pb);
    CG_LAUNCH_CHECK();
    bw_col_finalize_kernel<<<static_cast<int>(ceil_div(static_cast<int64_t>(d) * 32, 256)), 256, 0, s>>>(
        n, d, normalize ? 1 : 0, pa, pb, partial, A, B, scaled);
    CG_LAUNCH_CHECK();
    bw_apply_kernel<<<grid_of(n * d), 256, 0, s>>>(d_x, n, d, mean, inv, gxc, A, B, scaled, grad_x);
    CG_LAUNCH_CHECK();
}

}  // namespace culof_gb300
