// Preprocessing: centring / z-scoring and squared row norms.
//
// Reference: src/cuda/preprocess.cu:31-72 (standardize_kernel: FP64 mean and
// population std per feature, zero-variance features keep scale 1, x written
// back as float((x - mean) * inv_std)) and :75-84 (squared_norms_kernel: FP64
// sum of squares cast to float).
//
// The reference reduces each feature with one block (tree order). Here the
// reduction is split into partial sums over chunks of kCenterChunk rows, each
// summed sequentially in row order, and the partials are then summed in chunk
// order. That order is fixed and is the one the CPU oracle uses, so the FP64
// means (and the centred floats) agree with it bit for bit; the partials give
// n/kCenterChunk x d parallel work instead of d blocks.
#include "common.cuh"
#include "prep.cuh"

namespace culof_gb300 {

namespace {

// One thread per (chunk, feature). mean == nullptr: sums x; otherwise sums
// (x - mean)^2. Consecutive threads are consecutive features of the same
// rows, so each row read is coalesced across the feature threads.
__global__ void center_partials_kernel(const float* __restrict__ x, int64_t n, int d,
                                       const double* __restrict__ mean,
                                       double* __restrict__ partial) {
    const int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    const int64_t chunks = ceil_div(n, kCenterChunk);
    if (t >= chunks * d) return;
    const int64_t c = t / d;
    const int f = static_cast<int>(t % d);
    const int64_t begin = c * kCenterChunk;
    const int64_t end = begin + kCenterChunk < n ? begin + kCenterChunk : n;
    double s = 0.0;
    if (mean == nullptr) {
        for (int64_t i = begin; i < end; ++i) s = __dadd_rn(s, static_cast<double>(x[i * d + f]));
    } else {
        const double m = mean[f];
        for (int64_t i = begin; i < end; ++i) {
            const double v = __dsub_rn(static_cast<double>(x[i * d + f]), m);
            s = __dadd_rn(s, __dmul_rn(v, v));
        }
    }
    partial[t] = s;
}

// One block per feature: the feature's partials are staged in shared memory
// (the whole block loads, many loads in flight), then one thread sums them in
// chunk order. mode 0 -> mean[f]; mode 1 -> inv_std[f] (population std; 1 for
// sd <= 1e-12).
constexpr int kFinalizeBuf = 4096;
__global__ void center_finalize_kernel(const double* __restrict__ partial, int64_t chunks,
                                       int d, int64_t n, int mode, double* __restrict__ mean,
                                       double* __restrict__ inv_std) {
    __shared__ double buf[kFinalizeBuf];
    const int f = blockIdx.x;
    double total = 0.0;
    for (int64_t c0 = 0; c0 < chunks; c0 += kFinalizeBuf) {
        const int m = static_cast<int>(chunks - c0 < kFinalizeBuf ? chunks - c0 : kFinalizeBuf);
        for (int i = threadIdx.x; i < m; i += blockDim.x) buf[i] = partial[(c0 + i) * d + f];
        __syncthreads();
        if (threadIdx.x == 0)
            for (int i = 0; i < m; ++i) total = __dadd_rn(total, buf[i]);
        __syncthreads();
    }
    if (threadIdx.x != 0) return;
    const double dn = static_cast<double>(n);
    if (mode == 0) {
        mean[f] = __ddiv_rn(total, dn);
        inv_std[f] = 1.0;
    } else {
        const double sd = __dsqrt_rn(__ddiv_rn(total, dn));
        inv_std[f] = (sd > 1e-12) ? __ddiv_rn(1.0, sd) : 1.0;
    }
}

__global__ void center_apply_kernel(const float* __restrict__ x, int64_t n, int d,
                                    const double* __restrict__ mean,
                                    const double* __restrict__ inv_std,
                                    float* __restrict__ xc) {
    const int64_t total = n * d;
    for (int64_t t = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; t < total;
         t += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const int f = static_cast<int>(t % d);
        const double v = __dmul_rn(__dsub_rn(static_cast<double>(x[t]), mean[f]), inv_std[f]);
        xc[t] = __double2float_rn(v);
    }
}

// norms[i] = (float) sum_f (double) xc[i,f]^2 (feature order), and the
// maximum norm (non-negative float bits order like the values).
__global__ void norms_kernel(const float* __restrict__ xc, int64_t n, int d,
                             float* __restrict__ norms, unsigned int* __restrict__ max_norm_bits) {
    unsigned int local_max = 0u;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const float* row = xc + i * d;
        double s = 0.0;
        for (int f = 0; f < d; ++f) {
            const double v = static_cast<double>(row[f]);
            s = __dadd_rn(s, __dmul_rn(v, v));
        }
        const float nf = __double2float_rn(s);
        norms[i] = nf;
        local_max = max(local_max, __float_as_uint(nf));
    }
    if (max_norm_bits != nullptr) {
        for (int o = 16; o > 0; o >>= 1) local_max = max(local_max, __shfl_xor_sync(0xffffffffu, local_max, o));
        if ((threadIdx.x & 31) == 0) atomicMax(max_norm_bits, local_max);
    }
}

int grid_for(int64_t items, int block, int max_blocks = 152 * 16) {
    int64_t g = ceil_div(items, block);
    if (g < 1) g = 1;
    if (g > max_blocks) g = max_blocks;
    return static_cast<int>(g);
}

}  // namespace

void center(const float* x, int64_t n, int d, bool normalize, float* xc, double* partial,
            double* mean, double* inv_std, cudaStream_t s) {
    const int64_t chunks = ceil_div(n, kCenterChunk);
    const int64_t items = chunks * d;
    const int block = 256;
    const int pgrid = static_cast<int>(ceil_div(items, block));
    center_partials_kernel<<<pgrid, block, 0, s>>>(x, n, d, nullptr, partial);
    CG_LAUNCH_CHECK();
    center_finalize_kernel<<<d, 256, 0, s>>>(partial, chunks, d, n, 0, mean, inv_std);
    CG_LAUNCH_CHECK();
    if (normalize) {
        center_partials_kernel<<<pgrid, block, 0, s>>>(x, n, d, mean, partial);
        CG_LAUNCH_CHECK();
        center_finalize_kernel<<<d, 256, 0, s>>>(partial, chunks, d, n, 1, mean, inv_std);
        CG_LAUNCH_CHECK();
    }
    center_apply_kernel<<<grid_for(n * d, 256), 256, 0, s>>>(x, n, d, mean, inv_std, xc);
    CG_LAUNCH_CHECK();
}

void squared_norms(const float* xc, int64_t n, int d, float* norms, unsigned int* max_norm_bits,
                   cudaStream_t s) {
    if (max_norm_bits != nullptr) CG_CUDA(cudaMemsetAsync(max_norm_bits, 0, sizeof(unsigned int), s));
    norms_kernel<<<grid_for(n, 256), 256, 0, s>>>(xc, n, d, norms, max_norm_bits);
    CG_LAUNCH_CHECK();
}

size_t center_partial_count(int64_t n, int d) { return static_cast<size_t>(ceil_div(n, kCenterChunk)) * d; }

}  // namespace culof_gb300
