// Shared device/host helpers for the culof_gb300 engine (sm_103a only).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <stdexcept>
#include <string>

namespace culof_gb300 {

// Status codes of the C ABI (include/culof_c.h).
enum Status : int {
    kOk = 0,
    kInvalidArgument = 1,
    kCudaError = 2,
    kNoDevice = 3,
    kInternal = 4,
    kKernelFault = 5,  // a kernel reported an error word (bounded wait expired, bad state)
};

// Thrown inside the library; the C ABI converts it to a status + message.
struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

void throw_cuda(cudaError_t err, const char* file, int line, const char* expr);

#define CG_CUDA(expr)                                                                  \
    do {                                                                               \
        cudaError_t _e = (expr);                                                       \
        if (_e != cudaSuccess) ::culof_gb300::throw_cuda(_e, __FILE__, __LINE__, #expr); \
    } while (0)

// Every kernel launch of the library is followed by this check, which also
// counts the launch (culof_kernel_launch_count in the C ABI).
void count_launch();
void count_launches(unsigned long long n);
void uncount_launches(unsigned long long n);
#define CG_LAUNCH_CHECK()                  \
    do {                                   \
        ::culof_gb300::count_launch();     \
        CG_CUDA(cudaGetLastError());       \
    } while (0)

// Raise a kernel's dynamic shared-memory limit on the current device, once
// per (kernel, device) in the process (engine.cu).
void set_max_dynamic_smem(const void* kernel, int bytes);

// Selection keys: (squared-distance bits << 32) | original column index.
// Squared distances are never negative (and never -0.0), so their IEEE bit
// patterns order like the values; the index breaks ties in ascending order.
__host__ __device__ __forceinline__ uint64_t make_key(uint32_t d2_bits, uint32_t idx) {
    return (static_cast<uint64_t>(d2_bits) << 32) | idx;
}
__host__ __device__ __forceinline__ uint32_t key_bits(uint64_t key) {
    return static_cast<uint32_t>(key >> 32);
}
__host__ __device__ __forceinline__ uint32_t key_index(uint64_t key) {
    return static_cast<uint32_t>(key & 0xFFFFFFFFull);
}

constexpr uint64_t kKeyMax = ~0ull;

// Rows per partial sum of the centring reduction (the CPU oracle uses the same
// order, so the FP64 means agree bit for bit).
constexpr int kCenterChunk = 256;

__host__ __device__ inline int64_t ceil_div(int64_t a, int64_t b) { return (a + b - 1) / b; }

// Squared distance by direct differences, float32, fixed order:
// t = a_f - b_f (rounded), s = fma(t, t, s), f ascending from s = +0.
// Every path of the engine computes exact distances with this function (or
// a bit-identical unrolled copy), so all paths select the same neighbours.
__device__ __forceinline__ float dist2_direct(const float* __restrict__ a,
                                              const float* __restrict__ b, int d) {
    float s = 0.0f;
    for (int f = 0; f < d; ++f) {
        const float t = __fsub_rn(a[f], b[f]);
        s = __fmaf_rn(t, t, s);
    }
    return s;
}

}  // namespace culof_gb300
