// FP32 CUDA-core throughput probe: the roofline denominator of the distance
// sweep, which is FP32 FMA bound (no FP32 SIMT figure is published for
// GB300 in a form this project can cite, so it is measured).
//
// Each thread runs 8 independent FMA chains (scalar fma.rn.f32, or packed
// fma.rn.f32x2 = 2 FMAs per instruction) for `iters` rounds; the result is
// stored so nothing is eliminated. FLOP = 2 per FMA.
#include "../../include/culof_c.h"
#include "common.cuh"

namespace culof_gb300 {

namespace {

__global__ void ffma_probe_kernel(float* out, int iters, float a, float b) {
    float x[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) x[i] = threadIdx.x * 1e-7f + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) x[i] = __fmaf_rn(x[i], a, b);
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += x[i];
    if (s == 12345.678f) out[0] = s;  // practically never; keeps the chains live
}

__global__ void ffma2_probe_kernel(float* out, int iters, float a, float b) {
    unsigned long long x[8];
    const unsigned long long A = (static_cast<unsigned long long>(__float_as_uint(a)) << 32) | __float_as_uint(a);
    const unsigned long long B = (static_cast<unsigned long long>(__float_as_uint(b)) << 32) | __float_as_uint(b);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const float v = threadIdx.x * 1e-7f + i;
        x[i] = (static_cast<unsigned long long>(__float_as_uint(v + 0.5f)) << 32) | __float_as_uint(v);
    }
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) asm volatile("fma.rn.f32x2 %0, %0, %1, %2;" : "+l"(x[i]) : "l"(A), "l"(B));
    }
    float s = 0.0f;
#pragma unroll
    for (int i = 0; i < 8; ++i) s += __uint_as_float(static_cast<unsigned>(x[i])) + __uint_as_float(static_cast<unsigned>(x[i] >> 32));
    if (s == 12345.678f) out[0] = s;
}

}  // namespace

}  // namespace culof_gb300

extern "C" CULOF_API int culof_probe_fp32_tflops(int packed, double* tflops_out) {
    using namespace culof_gb300;
    if (tflops_out == nullptr) return CULOF_ERR_INVALID_ARGUMENT;
    try {
        int dev = 0, sms = 0;
        CG_CUDA(cudaGetDevice(&dev));
        CG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        float* out = nullptr;
        CG_CUDA(cudaMalloc(&out, sizeof(float)));
        cudaEvent_t e0, e1;
        CG_CUDA(cudaEventCreate(&e0));
        CG_CUDA(cudaEventCreate(&e1));
        const int blocks = sms * 8, threads = 256, iters = 1 << 14;
        double best = 0.0;
        for (int rep = 0; rep < 4; ++rep) {
            CG_CUDA(cudaEventRecord(e0));
            if (packed) ffma2_probe_kernel<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
            else ffma_probe_kernel<<<blocks, threads>>>(out, iters, 0.999f, 1e-3f);
            CG_CUDA(cudaGetLastError());
            CG_CUDA(cudaEventRecord(e1));
            CG_CUDA(cudaEventSynchronize(e1));
            float ms = 0.0f;
            CG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            const double fmas = static_cast<double>(blocks) * threads * iters * 8 * (packed ? 2 : 1);
            const double tf = 2.0 * fmas / (ms * 1e-3) / 1e12;
            if (rep > 0 && tf > best) best = tf;  // rep 0 warms up
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        cudaFree(out);
        *tflops_out = best;
        return CULOF_OK;
    } catch (const Error& e) {
        return e.status;
    }
}
