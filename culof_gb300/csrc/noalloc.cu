// culof_contamination_offset_noalloc: the contamination-offset select with no
// device allocation at all.
//
// Some callers cannot call cudaMalloc while they run: a GPU operator embedded
// in a host framework that owns every byte of device memory through its own
// pool and forbids driver allocations on its processing path (a cudaMalloc or
// cudaFree there can synchronise the whole device and fragments the pool), or
// a latency-bound loop that must never stall on an allocation. Such callers
// pass their own device buffers for the input and the output; the select's
// scratch (a 2048-bin histogram and a small state block) lives in the
// file-scope device array below, which every GPU that loads this library
// holds until the process exits.
//
// Set-up: the first call on a device looks up the array's device address
// with cudaGetSymbolAddress (with that device current) and caches it, so
// make that first call before any stream capture.
// Sharing: every call on a device uses the same array, which keeps the last
// call's contents; each call clears the histogram and state first. Calls that
// overlap on the GPU (e.g. on two streams at once) race on the array.
#include <mutex>
#include <sstream>
#include <string>

#include "../../include/culof_c.h"
#include "common.cuh"
#include "engine.cuh"
#include "prep.cuh"

namespace culof_gb300 {

void set_last_error(const std::string& msg);

namespace {

// Histogram bins + select state: 8,232 bytes.
constexpr size_t kNoAllocScratchBytes = kOffsetHistBins * sizeof(int) + sizeof(OffsetState);
static_assert(kNoAllocScratchBytes == 8232, "documented scratch size");
// The select counts points in 32-bit integers.
constexpr int64_t kNoAllocMaxPoints = 0x7FFFFFFF;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_offset_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_addr[kMaxDevices] = {};

// Device address of g_offset_scratch on the current device (set up once per
// device). In host code the array's name is only a host-side stand-in.
void* scratch_address() {
    int dev = 0;
    CG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw Error(kInternal, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (g_scratch_addr[dev] == nullptr) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_offset_scratch);
        if (e != cudaSuccess)
            throw Error(kCudaError, std::string("cudaGetSymbolAddress(offset scratch) failed: ") +
                                        cudaGetErrorString(e));
        g_scratch_addr[dev] = p;
    }
    return g_scratch_addr[dev];
}

}  // namespace
}  // namespace culof_gb300

extern "C" CULOF_API int culof_contamination_offset_noalloc(void* cuda_stream, const float* d_nof, int64_t n_points,
                                                            double contamination, double* d_offset) {
    using namespace culof_gb300;
    try {
        if (d_nof == nullptr || d_offset == nullptr) throw Error(kInvalidArgument, "device pointers must not be null");
        if (n_points < 1) throw Error(kInvalidArgument, "n_points must be >= 1");
        if (n_points > kNoAllocMaxPoints) {
            std::ostringstream os;
            os << "n_points must be at most " << kNoAllocMaxPoints << " for the allocation-free offset (got "
               << n_points << ")";
            throw Error(kInvalidArgument, os.str());
        }
        validate_contamination(contamination);
        void* scratch = scratch_address();
        contamination_offset(d_nof, n_points, plan_offset(n_points, contamination), scratch, d_offset,
                             static_cast<cudaStream_t>(cuda_stream));
        set_last_error("");
        return CULOF_OK;
    } catch (const Error& e) {
        set_last_error(e.what());
        return e.status;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return CULOF_ERR_INTERNAL;
    }
}
