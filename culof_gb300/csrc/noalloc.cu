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
// make that first call before any stream capture. The cache is keyed on the
// current CUDA context's unique id: a context that the caller's framework
// destroys and creates again (cudaDeviceReset) gets a fresh lookup on its
// first call, never the old context's address.
// The stream must belong to the current device.
// Sharing: every call on a device uses the same array, which keeps the last
// call's contents; each call clears the histogram and state first. Calls that
// overlap on the GPU (e.g. on two streams at once) race on the array.
#include <cuda.h>

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

struct ScratchSlot {
    void* addr = nullptr;
    unsigned long long context_id = 0;
};

std::mutex g_setup_mutex;
ScratchSlot g_scratch[kMaxDevices];

// Unique id of the calling thread's current CUDA context (0: none current, or
// the driver cannot say). The driver functions come through the runtime's
// entry-point query, so the library needs no link to the driver library.
unsigned long long current_context_id() {
    using GetCurrentFn = CUresult (*)(CUcontext*);
    using GetIdFn = CUresult (*)(CUcontext, unsigned long long*);
    static GetCurrentFn get_current = nullptr;
    static GetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* f = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_current = reinterpret_cast<GetCurrentFn>(f);
        f = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<GetIdFn>(f);
    });
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (!get_current || !get_id || get_current(&ctx) != CUDA_SUCCESS || ctx == nullptr) return 0;
    if (get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of g_offset_scratch in the current device's context, looked
// up once per (device, context). In host code the array's name is only a
// host-side stand-in, never a device address.
void* scratch_address() {
    int dev = 0;
    CG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kMaxDevices) throw Error(kInternal, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    ScratchSlot& slot = g_scratch[dev];
    const unsigned long long ctx = current_context_id();
    if (slot.addr == nullptr || ctx == 0 || slot.context_id != ctx) {
        void* p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_offset_scratch);
        if (e != cudaSuccess)
            throw Error(kCudaError, std::string("cudaGetSymbolAddress(offset scratch) failed: ") +
                                        cudaGetErrorString(e));
        slot.addr = p;
        // the lookup makes the device's context current if none was
        slot.context_id = current_context_id();
    }
    return slot.addr;
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
