// Pipeline orchestration (the reference's culof::lof, pipeline.cu:131-207),
// re-planned around a persistent context: one stream and grow-only
// workspaces per context instead of seven cudaMallocs and a stream per call,
// no cuBLAS, and a fused k-NN path whose n x n distances never reach HBM.
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <mutex>
#include <set>
#include <sstream>
#include <utility>

#include "engine.cuh"
#include "fast.cuh"
#include "sweep_common.cuh"
#include "tc_host.cuh"

namespace culof_gb300 {

namespace {
std::atomic<unsigned long long> g_launches{0};

// A wait on an mbarrier phase that nothing completes, bounded like every
// wait of the engine's kernels: after `limit` polls it gives up, sets the
// status word and returns, so the context stays usable.
__global__ void wait_probe_kernel(int* status, long long limit) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        sweep::mbar_init(&bar, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    if (threadIdx.x == 0 && !sweep::mbar_wait(&bar, 0, limit)) atomicExch(status, 1);
}
}  // namespace

void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void count_launches(unsigned long long n) { g_launches.fetch_add(n, std::memory_order_relaxed); }
void uncount_launches(unsigned long long n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }
unsigned long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

void set_max_dynamic_smem(const void* kernel, int bytes) {
    static std::mutex mu;
    static std::set<std::pair<std::pair<const void*, int>, int>> done;  // ((kernel, device), bytes)
    int dev = 0;
    CG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lock(mu);
    if (done.count({{kernel, dev}, bytes})) return;
    CG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
    done.insert({{kernel, dev}, bytes});
}

void throw_cuda(cudaError_t err, const char* file, int line, const char* expr) {
    std::ostringstream os;
    os << "CUDA error at " << file << ":" << line << " (" << expr << "): " << cudaGetErrorString(err);
    throw Error(kCudaError, os.str());
}

void* DevBuf::get(size_t bytes) {
    if (bytes == 0) bytes = 16;
    if (bytes > cap_) {
        release();
        // Round up so slowly growing problem sizes do not reallocate every call.
        size_t want = bytes + bytes / 8;
        want = (want + 255) & ~static_cast<size_t>(255);
        CG_CUDA(cudaMalloc(&ptr_, want));
        cap_ = want;
    }
    return ptr_;
}

void DevBuf::release() {
    if (ptr_) cudaFree(ptr_);
    ptr_ = nullptr;
    cap_ = 0;
}

void validate_lof_args(const void* points, int64_t n, int d, int k) {
    if (points == nullptr) throw Error(kInvalidArgument, "points must not be null");
    if (n < 2) throw Error(kInvalidArgument, "n_points must be >= 2");
    if (d < 1) throw Error(kInvalidArgument, "n_dims must be >= 1");
    if (k < 1 || static_cast<int64_t>(k) >= n) {
        std::ostringstream os;
        os << "k must satisfy 1 <= k <= n_points - 1 (got k=" << k << ", n_points=" << n << ")";
        throw Error(kInvalidArgument, os.str());
    }
    if (n > 0x7FFFFFFFll) throw Error(kInvalidArgument, "n_points must be < 2^31");
}

void validate_contamination(double c) {
    if (c > 0.5 || c != c) {
        std::ostringstream os;
        os << "contamination must be 'auto' or in (0, 0.5], got " << c;
        throw Error(kInvalidArgument, os.str());
    }
}

Engine::Engine(int device) : device_(device) {
    CG_CUDA(cudaSetDevice(device_));
    // A blocking stream (as pipeline.cu:64 creates): it orders with work on
    // the legacy default stream, which callers' frameworks often use.
    CG_CUDA(cudaStreamCreate(&own_stream_));
    stream_ = own_stream_;
    CG_CUDA(cudaMemset(status_ptr(), 0, sizeof(int)));
}

Engine::~Engine() {
    if (bgraph_exec_) cudaGraphExecDestroy(bgraph_exec_);
    for (auto& e : events_)
        if (e) cudaEventDestroy(e);
    for (cudaStream_t st : {high_stream_, side_stream_})
        if (st) {
            cudaSetDevice(device_);
            cudaStreamSynchronize(st);
            cudaStreamDestroy(st);
        }
    for (cudaEvent_t e : {fork_ev_, high_join_, side_join_})
        if (e) cudaEventDestroy(e);
    if (own_stream_) {
        cudaSetDevice(device_);
        cudaStreamSynchronize(own_stream_);
        cudaStreamDestroy(own_stream_);
    }
}

void Engine::make_fork_streams() {
    if (side_stream_) return;
    // non-blocking (they must not wait for the legacy default stream); the
    // high one of the greatest priority, the side one of the least, so that
    // of two kernels that become ready together the high one's CTAs are
    // dispatched first
    int least = 0, greatest = 0;
    CG_CUDA(cudaDeviceGetStreamPriorityRange(&least, &greatest));
    CG_CUDA(cudaStreamCreateWithPriority(&high_stream_, cudaStreamNonBlocking, greatest));
    CG_CUDA(cudaStreamCreateWithPriority(&side_stream_, cudaStreamNonBlocking, least));
    for (cudaEvent_t* e : {&fork_ev_, &high_join_, &side_join_})
        CG_CUDA(cudaEventCreateWithFlags(e, cudaEventDisableTiming));
}

// pipeline.cu:99-110: CULOF_TILE_ROWS overrides; otherwise a 2 GiB cap on
// free memory less a 128 MiB margin.
int Engine::tile_rows_for(int64_t n) {
    if (const char* env = std::getenv("CULOF_TILE_ROWS")) {
        const long forced = std::atol(env);
        if (forced > 0) return static_cast<int>(forced < n ? forced : n);
    }
    size_t free_b = 0, total_b = 0;
    CG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t cap = size_t(2) << 30, margin = size_t(128) << 20;
    const size_t usable = free_b > margin ? free_b - margin : 0;
    return choose_tile_rows(n, usable < cap ? usable : cap);
}

// AUTO: the general tile + select path for n <= 4096 (a few kernels against
// the fused paths' ~45; fit_predict on the device, d = 8, k = 20: n = 1000,
// 0.18 ms against 0.38 ms; n = 4000, 0.39 against 0.58 ms; n = 8000, 1.02
// against 0.62 ms) and beyond the fused paths' limits (d > 128 or k > 64);
// otherwise the FP32 fused
// sweep for d <= 8 and the tensor-core sweep for 8 < d <= 128 (the FP32 wide
// sweep for d <= 16 below one wave of row tiles). All give the same bits.
// CULOF_GB300_PATH=general|fast|tensor overrides AUTO for a process.
constexpr int64_t kSmallN = 4096;
int Engine::choose_path(int64_t n, int d, int k) const {
    int p = path_;
    if (p == kPathAuto) {
        if (const char* env = std::getenv("CULOF_GB300_PATH")) {
            if (env[0] == 'g') p = kPathGeneral;
            if (env[0] == 'f') p = kPathFast;
            if (env[0] == 't') p = kPathTensor;
        }
    }
    const bool ok = fast_path_supported(n, d, k);
    if (p == kPathGeneral) return kPathGeneral;
    if ((p == kPathFast || p == kPathTensor) && !ok)
        throw Error(kInvalidArgument, "fused path requested but unsupported for this n/d/k");
    if (p == kPathFast || p == kPathTensor) return p;
    if (!ok || n <= kSmallN) return kPathGeneral;
    // d <= 8: the FP32 small-d sweep at every k (fit_predict on clusters
    // against the tensor sweep over the same seed window and prune lists:
    // k = 64, n = 20k / 50k / 200k: 1.42 / 3.13 / 17.6 against 3.38 / 6.90 /
    // 25.2 ms; k = 48, 200k: 16.3 against 18.8 ms)
    if (d <= 8) return kPathFast;
    // 8 < d <= 16 with fewer row tiles than SMs: the FP32 wide sweep ties the
    // tensor path (n = 20k, d = 16: 1.91 against 1.87 ms); from there up the
    // tensor path wins (n = 30k: 2.33 against 2.80 ms; 38k: 3.01 against
    // 3.79 ms), and at every size for d > 16 (d = 24, n = 20k: 1.81 against
    // 2.31 ms; d = 32, n = 10k: 1.15 against 1.45 ms)
    int sms = 0;
    CG_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device_));
    const int64_t nt = (n + 127) / 128;
    if (d <= 16 && nt < static_cast<int64_t>(sms)) return kPathFast;
    return kPathTensor;
}

void Engine::knn_general(const float* xc, const float* norms, int64_t n, int d, int k,
                         int32_t* nbr_idx, float* nbr_d2, float* kdist2, int64_t row_begin, int64_t row_end) {
    const int tile = tile_rows_for(n);
    float* d_tile = tile_.as<float>(static_cast<size_t>(tile) * n);
    for (int64_t row0 = row_begin; row0 < row_end; row0 += tile) {
        const int rows = static_cast<int>((row_end - row0) < tile ? (row_end - row0) : tile);
        distance_tile(xc, n, d, row0, rows, d_tile, stream_);
        select_tile_rows(d_tile, norms, rows, row0, n, k, kSelectDistances, nbr_idx, nbr_d2, kdist2, stream_);
    }
}

void Engine::knn(const float* d_x, int64_t n, int d, int k, bool normalize, int32_t* nbr_idx,
                 float* nbr_d2, float* kdist2) {
    knn_core(d_x, n, d, k, normalize, 0, 1, nbr_idx, nbr_d2, kdist2, nullptr);
}

int64_t Engine::knn_shard(const float* d_x, int64_t n, int d, int k, bool normalize, int shard, int num_shards,
                          int32_t* nbr_idx, float* nbr_d2, float* kdist2, int32_t* rows) {
    if (num_shards < 1 || shard < 0 || shard >= num_shards)
        throw Error(kInvalidArgument, "shard must satisfy 0 <= shard < num_shards");
    if (rows == nullptr) throw Error(kInvalidArgument, "rows must not be null");
    return knn_core(d_x, n, d, k, normalize, shard, num_shards, nbr_idx, nbr_d2, kdist2, rows);
}

int64_t Engine::knn_core(const float* d_x, int64_t n, int d, int k, bool normalize, int shard, int num_shards,
                         int32_t* nbr_idx, float* nbr_d2, float* kdist2, int32_t* rows) {
    validate_lof_args(d_x, n, d, k);
    CG_CUDA(cudaSetDevice(device_));
    float* xc = xc_.as<float>(static_cast<size_t>(n) * d);
    double* partial = partial_.as<double>(center_partial_count(n, d));
    double* mean = mean_.as<double>(d);
    double* inv = inv_std_.as<double>(d);
    float* norms = norms_.as<float>(n);
    unsigned int* maxn = max_norm_.as<unsigned int>(1);
    CG_CUDA(cudaMemsetAsync(status_ptr(), 0, sizeof(int), stream_));
    stat_total_blocks_ = 0;
    for (bool& m : marked_) m = false;
    mark(0);
    center(d_x, n, d, normalize, xc, partial, mean, inv, stream_);
    squared_norms(xc, n, d, norms, maxn, stream_);
    const int path = choose_path(n, d, k);
    int64_t count = n;
    if (path != kPathGeneral) {
        last_path_ = path;
        mark(1);
        knn_fast(xc, norms, n, d, k, path == kPathTensor, nbr_idx, nbr_d2, kdist2, shard, num_shards, rows);
        if (num_shards > 1) {  // whole row tiles of 128 points
            const int64_t nt = (n + 127) / 128;
            const int64_t t0 = nt * shard / num_shards, t1 = nt * (shard + 1) / num_shards;
            count = std::min<int64_t>(n, t1 * 128) - std::min<int64_t>(n, t0 * 128);
        }
    } else {
        last_path_ = kPathGeneral;
        mark(1);
        mark(2);
        mark(3);
        // a shard of the general path: a block of original rows
        const int64_t b = n * shard / num_shards, e = n * (shard + 1) / num_shards;
        knn_general(xc, norms, n, d, k, nbr_idx, nbr_d2, kdist2, b, e);
        if (rows && e > b) iota_rows(rows, b, e - b, stream_);
        count = e - b;
        mark(4);
    }
    mark(5);
    return count;
}

void Engine::lof_device(const float* d_x, int64_t n, int d, int k, bool normalize, float* d_scores,
                        float* d_nof) {
    validate_lof_args(d_x, n, d, k);
    const size_t nk = static_cast<size_t>(n) * k;
    int32_t* idx = nbr_idx_.as<int32_t>(nk);
    float* d2 = nbr_d2_.as<float>(nk);
    float* kd = kdist2_.as<float>(n);
    float* lrd = lrd_.as<float>(n);
    knn(d_x, n, d, k, normalize, idx, d2, kd);
    compute_lrd(idx, d2, kd, n, k, lrd, status_ptr(), stream_);
    compute_scores(idx, lrd, n, k, d_scores, d_nof, status_ptr(), stream_);
    mark(6);
}

void Engine::offset_device(const float* d_nof, int64_t n, double contamination, double* d_offset) {
    validate_contamination(contamination);
    void* scratch = offset_scratch_.get(offset_scratch_bytes());
    contamination_offset(d_nof, n, plan_offset(n, contamination), scratch, d_offset, stream_);
}

void Engine::bf16_gram(const void* A, int64_t rows_a, const void* B, int64_t rows_b, int K, float* G) {
    CG_CUDA(cudaSetDevice(device_));
    tc::bf16_gram(A, rows_a, B, rows_b, K, G, status_ptr(), stream_);
}

void Engine::fit_predict_device(const float* d_x, int64_t n, int d, int k, bool normalize,
                                double contamination, float* d_nof, int64_t* d_labels,
                                double* d_offset) {
    validate_lof_args(d_x, n, d, k);
    validate_contamination(contamination);
    float* scores = scores_.as<float>(n);
    float* nof = d_nof ? d_nof : nof_.as<float>(n);
    double* off = d_offset ? d_offset : offset_.as<double>(1);
    lof_device(d_x, n, d, k, normalize, scores, nof);
    offset_device(nof, n, contamination, off);
    if (d_labels) labels_from_offset(nof, n, off, d_labels, stream_);
    mark(7);
}

void Engine::lof_host(const float* x, int64_t n, int d, int k, bool normalize, float* scores) {
    validate_lof_args(x, n, d, k);
    if (scores == nullptr) throw Error(kInvalidArgument, "scores_out must not be null");
    CG_CUDA(cudaSetDevice(device_));
    float* dx = x_.as<float>(static_cast<size_t>(n) * d);
    float* ds = scores_.as<float>(n);
    CG_CUDA(cudaMemcpyAsync(dx, x, sizeof(float) * n * d, cudaMemcpyHostToDevice, stream_));
    lof_device(dx, n, d, k, normalize, ds, nullptr);
    CG_CUDA(cudaMemcpyAsync(scores, ds, sizeof(float) * n, cudaMemcpyDeviceToHost, stream_));
    check_status();
}

void Engine::set_timing(bool on) {
    if (on && !events_[0]) {
        CG_CUDA(cudaSetDevice(device_));
        for (auto& e : events_) CG_CUDA(cudaEventCreate(&e));
    }
    timing_ = on;
}

void Engine::mark(int boundary) {
    if (!timing_) return;
    CG_CUDA(cudaEventRecord(events_[boundary], stream_));
    marked_[boundary] = true;
}

void Engine::stage_times(float* ms, int cap) {
    CG_CUDA(cudaStreamSynchronize(stream_));
    for (int i = 0; i < kNumStages && i < cap; ++i) {
        ms[i] = -1.0f;
        if (timing_ && marked_[i] && marked_[i + 1]) CG_CUDA(cudaEventElapsedTime(&ms[i], events_[i], events_[i + 1]));
    }
}

void Engine::pair_stats(double* evaluated, double* total) {
    unsigned long long ev = 0;
    if (stat_total_blocks_ > 0) {
        CG_CUDA(cudaMemcpyAsync(&ev, pair_stats_.get(2 * sizeof(unsigned long long)), sizeof(ev),
                                cudaMemcpyDeviceToHost, stream_));
        CG_CUDA(cudaStreamSynchronize(stream_));
    }
    // one block = 16 rows x 128 columns
    if (evaluated) *evaluated = static_cast<double>(ev) * 16.0 * 128.0;
    if (total) *total = static_cast<double>(stat_total_blocks_) * 16.0 * 128.0;
}

void Engine::probe_bounded_wait(long long limit) {
    if (limit < 1 || limit > sweep::kSpinLimit) throw Error(kInvalidArgument, "spin limit out of range");
    CG_CUDA(cudaSetDevice(device_));
    CG_CUDA(cudaMemsetAsync(status_ptr(), 0, sizeof(int), stream_));
    wait_probe_kernel<<<1, 32, 0, stream_>>>(status_ptr(), limit);
    CG_LAUNCH_CHECK();
    check_status();
}

void Engine::check_status() {
    int st = 0;
    CG_CUDA(cudaMemcpyAsync(&st, status_ptr(), sizeof(int), cudaMemcpyDeviceToHost, stream_));
    CG_CUDA(cudaStreamSynchronize(stream_));
    if (st == 1) throw Error(kKernelFault, "k-NN kernel: a bounded wait on a tile copy expired");
    if (st != 0) throw Error(kKernelFault, "k-NN kernel produced an invalid neighbour index");
}

void Engine::fit_predict_host(const float* x, int64_t n, int d, int k, bool normalize,
                              double contamination, float* nof, int64_t* labels, double* offset) {
    validate_lof_args(x, n, d, k);
    validate_contamination(contamination);
    CG_CUDA(cudaSetDevice(device_));
    float* dx = x_.as<float>(static_cast<size_t>(n) * d);
    float* dnof = nof_.as<float>(n);
    int64_t* dlab = labels ? labels_.as<int64_t>(n) : nullptr;
    double* doff = offset_.as<double>(1);
    CG_CUDA(cudaMemcpyAsync(dx, x, sizeof(float) * n * d, cudaMemcpyHostToDevice, stream_));
    fit_predict_device(dx, n, d, k, normalize, contamination, dnof, dlab, doff);
    if (nof) CG_CUDA(cudaMemcpyAsync(nof, dnof, sizeof(float) * n, cudaMemcpyDeviceToHost, stream_));
    if (labels) CG_CUDA(cudaMemcpyAsync(labels, dlab, sizeof(int64_t) * n, cudaMemcpyDeviceToHost, stream_));
    double off_h = 0.0;
    CG_CUDA(cudaMemcpyAsync(&off_h, doff, sizeof(double), cudaMemcpyDeviceToHost, stream_));
    check_status();
    if (offset) *offset = off_h;
}

}  // namespace culof_gb300
