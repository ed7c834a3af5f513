// Local reachability density, LOF scores, the contamination offset and the
// labels.
//
// lrd / score follow src/cuda/lof.cu:32-62 term for term: FP64 sums in slot
// order, sqrt of the max of squared distances, the 1e-10 guard, float results.
// The offset replaces the host-side np.percentile of src/culof/__init__.py:183
// with a GPU order-statistic select plus numpy's 'linear' interpolation; the
// labels are predict()'s `nof < offset_` (__init__.py:208-210).
#include <cmath>

#include "block.cuh"
#include "common.cuh"
#include "prep.cuh"

namespace culof_gb300 {

namespace {

constexpr int kBlock = 256;

// One thread per point; `rows` (nullable) lists the m points of a row block
// (a shard of a row-sharded run), otherwise every point.
__device__ __forceinline__ int64_t block_row(const int32_t* rows, int64_t m, int64_t n, int* status) {
    const int64_t r = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= m) return -1;
    const int64_t i = rows ? static_cast<int64_t>(rows[r]) : r;
    if (i < 0 || i >= n) {
        if (status != nullptr) atomicExch(status, 2);
        return -1;
    }
    return i;
}

__global__ void lrd_kernel(const int32_t* __restrict__ nbr_idx, const float* __restrict__ nbr_d2,
                           const float* __restrict__ kdist2, int64_t n, int k, const int32_t* __restrict__ rows,
                           int64_t m, float* __restrict__ lrd, int* status) {
    const int64_t i = block_row(rows, m, n, status);
    if (i < 0) return;
    if (status != nullptr && *status != 0) {
        lrd[i] = __int_as_float(0x7fc00000);
        return;
    }
    double sum = 0.0;
    for (int t = 0; t < k; ++t) {
        const int64_t o = static_cast<int64_t>(t) * n + i;
        const int32_t j = nbr_idx[o];
        if (j < 0 || j >= n) {  // never happens for a valid k-NN graph; do not read out of range
            if (status != nullptr) atomicExch(status, 2);
            lrd[i] = __int_as_float(0x7fc00000);
            return;
        }
        sum = __dadd_rn(sum, __dsqrt_rn(static_cast<double>(fmaxf(kdist2[j], nbr_d2[o]))));
    }
    lrd[i] = __double2float_rn(__ddiv_rn(1.0, __dadd_rn(__ddiv_rn(sum, static_cast<double>(k)), 1e-10)));
}

__global__ void score_kernel(const int32_t* __restrict__ nbr_idx, const float* __restrict__ lrd,
                             int64_t n, int k, const int32_t* __restrict__ rows, int64_t m,
                             float* __restrict__ scores, float* __restrict__ nof, int* status) {
    const int64_t i = block_row(rows, m, n, status);
    if (i < 0) return;
    const double self = static_cast<double>(lrd[i]);
    double sum = 0.0;
    for (int t = 0; t < k; ++t) {
        const int32_t j = nbr_idx[static_cast<int64_t>(t) * n + i];
        if (j < 0 || j >= n) {
            if (status != nullptr) atomicExch(status, 2);
            sum = __longlong_as_double(0x7ff8000000000000ll);
            break;
        }
        sum = __dadd_rn(sum, __ddiv_rn(static_cast<double>(lrd[j]), self));
    }
    const float s = __double2float_rn(__ddiv_rn(sum, static_cast<double>(k)));
    scores[i] = s;
    if (nof != nullptr) nof[i] = -s;
}

// ---- contamination offset --------------------------------------------------

// Float -> uint32 whose unsigned order is the float order (negatives flipped).
__device__ __forceinline__ unsigned int order_key(float f) {
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float from_order_key(unsigned int k) {
    const unsigned int u = (k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k;
    return __uint_as_float(u);
}

__global__ void offset_init_kernel(int* __restrict__ hist, OffsetState* __restrict__ st) {
    for (int b = threadIdx.x; b < kOffsetHistBins; b += blockDim.x) hist[b] = 0;
    if (threadIdx.x == 0) {
        st->prefix = 0u;
        st->below = 0;
        st->a_key = 0u;
        st->min_gt = 0xFFFFFFFFu;
        st->count_le = 0;
        st->offset = 0.0;
        st->offset_f = 0.0f;
    }
}

// Histogram of the digit (shift, width) of every key whose bits above the
// digit equal the prefix found so far.
__global__ void offset_hist_kernel(const float* __restrict__ nof, int64_t n, int shift, int width,
                                   int* __restrict__ hist, const OffsetState* __restrict__ st) {
    __shared__ int sh[kOffsetHistBins];
    const int bins = 1 << width;
    for (int b = threadIdx.x; b < bins; b += blockDim.x) sh[b] = 0;
    __syncthreads();
    const unsigned int hi_mask = (shift + width >= 32) ? 0u : (0xFFFFFFFFu << (shift + width));
    const unsigned int prefix = st->prefix;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const unsigned int key = order_key(nof[i]);
        if ((key & hi_mask) == (prefix & hi_mask)) atomicAdd(&sh[(key >> shift) & (bins - 1)], 1);
    }
    __syncthreads();
    for (int b = threadIdx.x; b < bins; b += blockDim.x)
        if (sh[b]) atomicAdd(&hist[b], sh[b]);
}

// Single block: locate the bin of the need-th key, extend the prefix, and
// clear the histogram for the next pass.
__global__ void offset_pick_kernel(int* __restrict__ hist, int shift, int width, int64_t rank,
                                   OffsetState* __restrict__ st) {
    __shared__ int warp_sums[kBlock / 32];
    __shared__ int found_bin, found_acc;
    const int bins = 1 << width;
    const int per = bins / kBlock;
    const int need = static_cast<int>(rank + 1) - st->below;
    int local = 0;
    for (int b = threadIdx.x * per; b < (threadIdx.x + 1) * per; ++b) local += hist[b];
    int total;
    const int excl = block_exclusive_scan(local, warp_sums, total);
    if (excl < need && excl + local >= need) {
        int acc = excl, bin = threadIdx.x * per;
        for (int b = threadIdx.x * per; b < (threadIdx.x + 1) * per; ++b) {
            if (acc + hist[b] >= need) {
                bin = b;
                break;
            }
            acc += hist[b];
        }
        found_bin = bin;
        found_acc = acc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        st->prefix |= static_cast<unsigned int>(found_bin) << shift;
        st->below += found_acc;
    }
    for (int b = threadIdx.x; b < kOffsetHistBins; b += blockDim.x) hist[b] = 0;
}

// count of keys <= a, and the smallest key > a.
__global__ void offset_next_kernel(const float* __restrict__ nof, int64_t n, OffsetState* __restrict__ st) {
    const unsigned int a = st->prefix;
    int cnt = 0;
    unsigned int mn = 0xFFFFFFFFu;
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x) {
        const unsigned int key = order_key(nof[i]);
        if (key <= a) ++cnt;
        else mn = min(mn, key);
    }
    for (int o = 16; o > 0; o >>= 1) {
        cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
        mn = min(mn, __shfl_xor_sync(0xffffffffu, mn, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(&st->count_le, cnt);
        atomicMin(&st->min_gt, mn);
    }
}

__global__ void offset_finalize_kernel(int64_t lo, int use_upper, float w, int is_auto,
                                       OffsetState* __restrict__ st, double* __restrict__ out) {
    float r;
    if (is_auto) {
        r = -1.5f;
    } else {
        const unsigned int ak = st->prefix;
        const float a = from_order_key(ak);
        const float b = (static_cast<int64_t>(st->count_le) >= lo + 2) ? a : from_order_key(st->min_gt);
        const float diff = __fsub_rn(b, a);
        r = use_upper ? __fsub_rn(b, __fmul_rn(diff, w)) : __fadd_rn(a, __fmul_rn(diff, w));
    }
    st->a_key = st->prefix;
    st->offset_f = r;
    st->offset = static_cast<double>(r);
    *out = static_cast<double>(r);
}

__global__ void labels_kernel(const float* __restrict__ nof, int64_t n, const double* __restrict__ offset,
                              int64_t* __restrict__ labels) {
    const float off = __double2float_rn(*offset);
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<int64_t>(gridDim.x) * blockDim.x)
        labels[i] = nof[i] < off ? -1 : 1;
}

int small_grid(int64_t n) {
    int64_t g = ceil_div(n, kBlock);
    if (g > 152 * 4) g = 152 * 4;
    return static_cast<int>(g < 1 ? 1 : g);
}

}  // namespace

void compute_lrd(const int32_t* nbr_idx, const float* nbr_d2, const float* kdist2, int64_t n, int k,
                 float* lrd, int* status, cudaStream_t s, const int32_t* rows, int64_t m) {
    if (!rows) m = n;
    if (m <= 0) return;
    lrd_kernel<<<static_cast<unsigned>(ceil_div(m, kBlock)), kBlock, 0, s>>>(nbr_idx, nbr_d2, kdist2, n, k, rows, m,
                                                                             lrd, status);
    CG_LAUNCH_CHECK();
}

void compute_scores(const int32_t* nbr_idx, const float* lrd, int64_t n, int k, float* scores,
                    float* nof, int* status, cudaStream_t s, const int32_t* rows, int64_t m) {
    if (!rows) m = n;
    if (m <= 0) return;
    score_kernel<<<static_cast<unsigned>(ceil_div(m, kBlock)), kBlock, 0, s>>>(nbr_idx, lrd, n, k, rows, m, scores,
                                                                               nof, status);
    CG_LAUNCH_CHECK();
}

// numpy 'linear' percentile of a float32 array with a Python-float q as the
// reference's LOF.fit passes it (np.percentile(nof, 100.0 * c)):
// q = (100 c) / 100, v = (n - 1) q, lo = floor(v), gamma = v - lo; the
// interpolation itself runs in float32 (offset_finalize_kernel).
OffsetPlan plan_offset(int64_t n, double contamination) {
    OffsetPlan p{};
    if (contamination <= 0.0) {
        p.is_auto = 1;
        return p;
    }
    const double q = (100.0 * contamination) / 100.0;
    const double v = static_cast<double>(n - 1) * q;
    double lo = std::floor(v);
    if (v >= static_cast<double>(n - 1)) lo = static_cast<double>(n - 1);
    if (lo < 0) lo = 0;
    const double gamma = v - lo;
    p.lo = static_cast<int64_t>(lo);
    p.use_upper = gamma >= 0.5 ? 1 : 0;
    p.w = p.use_upper ? static_cast<float>(1.0 - gamma) : static_cast<float>(gamma);
    if (p.lo >= n - 1) {  // no upper neighbour: the largest value itself
        p.lo = n - 1;
        p.use_upper = 0;
        p.w = 0.0f;
    }
    return p;
}

size_t offset_scratch_bytes() { return kOffsetHistBins * sizeof(int) + sizeof(OffsetState); }

void contamination_offset(const float* nof, int64_t n, const OffsetPlan& plan, void* scratch,
                          double* offset_out_dev, cudaStream_t s) {
    int* hist = static_cast<int*>(scratch);
    OffsetState* st = reinterpret_cast<OffsetState*>(hist + kOffsetHistBins);
    offset_init_kernel<<<1, kBlock, 0, s>>>(hist, st);
    CG_LAUNCH_CHECK();
    if (!plan.is_auto) {
        const int g = small_grid(n);
        const int shifts[3] = {21, 10, 0}, widths[3] = {11, 11, 10};
        for (int p = 0; p < 3; ++p) {
            offset_hist_kernel<<<g, kBlock, 0, s>>>(nof, n, shifts[p], widths[p], hist, st);
            CG_LAUNCH_CHECK();
            offset_pick_kernel<<<1, kBlock, 0, s>>>(hist, shifts[p], widths[p], plan.lo, st);
            CG_LAUNCH_CHECK();
        }
        offset_next_kernel<<<g, kBlock, 0, s>>>(nof, n, st);
        CG_LAUNCH_CHECK();
    }
    offset_finalize_kernel<<<1, 1, 0, s>>>(plan.lo, plan.use_upper, plan.w, plan.is_auto, st, offset_out_dev);
    CG_LAUNCH_CHECK();
}

void labels_from_offset(const float* nof, int64_t n, const double* offset_dev, int64_t* labels,
                        cudaStream_t s) {
    labels_kernel<<<small_grid(n), kBlock, 0, s>>>(nof, n, offset_dev, labels);
    CG_LAUNCH_CHECK();
}

}  // namespace culof_gb300
