// The C ABI (include/culof_c.h) and the C++ API (include/culof.h) over the
// engine. Exceptions never cross the C ABI: every entry point converts them
// into a status code and a per-thread message.
#include <cstdio>
#include <cstring>
#include <memory>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/culof.h"
#include "../../include/culof_c.h"
#include "engine.cuh"

struct culof_context {
    std::unique_ptr<culof_gb300::Engine> engine;
};

namespace {

using culof_gb300::Engine;
using culof_gb300::Error;

thread_local std::string g_last_error;

template <typename F>
int guarded(F&& f) {
    try {
        f();
        g_last_error.clear();
        return CULOF_OK;
    } catch (const Error& e) {
        g_last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        g_last_error = "host allocation failed";
        return CULOF_ERR_INTERNAL;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return CULOF_ERR_INTERNAL;
    }
}

bool device_present() {
    int count = 0;
    return cudaGetDeviceCount(&count) == cudaSuccess && count > 0;
}

void require_device() {
    if (!device_present()) throw Error(culof_gb300::kNoDevice, "no CUDA device available");
}

// One default context per thread and device, created on first use (the
// reference keeps one cuBLAS handle per thread for the same reason,
// pipeline.cu:76-87).
Engine& thread_engine() {
    thread_local std::unique_ptr<Engine> eng;
    int dev = 0;
    CG_CUDA(cudaGetDevice(&dev));
    if (!eng || eng->device() != dev) eng.reset(new Engine(dev));
    return *eng;
}

Engine& engine_of(culof_context* ctx) {
    if (ctx == nullptr || !ctx->engine) throw Error(culof_gb300::kInvalidArgument, "context must not be null");
    return *ctx->engine;
}

}  // namespace

namespace culof_gb300 {
// Lets entry points defined in other files report through culof_last_error().
void set_last_error(const std::string& msg) { g_last_error = msg; }
}  // namespace culof_gb300

extern "C" {

const char* culof_version(void) { return "0.2.0"; }

const char* culof_last_error(void) { return g_last_error.c_str(); }

int culof_cuda_available(void) { return device_present() ? 1 : 0; }

int culof_device_info(char* buf, size_t cap) {
    return guarded([&] {
        if (buf == nullptr || cap == 0) throw Error(culof_gb300::kInvalidArgument, "buffer must not be empty");
        std::string s;
        int device = 0;
        cudaDeviceProp prop{};
        if (cudaGetDevice(&device) != cudaSuccess) {
            s = "no CUDA device";
        } else if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
            s = "unknown device";
        } else {
            std::ostringstream os;
            os << prop.name << " (sm_" << prop.major << prop.minor << ", " << prop.multiProcessorCount
               << " SMs, " << (prop.totalGlobalMem >> 20) << " MiB)";
            s = os.str();
        }
        std::snprintf(buf, cap, "%s", s.c_str());
    });
}

int culof_context_create(culof_context** out) {
    return guarded([&] {
        if (out == nullptr) throw Error(culof_gb300::kInvalidArgument, "out must not be null");
        *out = nullptr;
        require_device();
        int dev = 0;
        CG_CUDA(cudaGetDevice(&dev));
        std::unique_ptr<culof_context> c(new culof_context);
        c->engine.reset(new Engine(dev));
        *out = c.release();
    });
}

void culof_context_destroy(culof_context* ctx) { delete ctx; }

int culof_context_set_stream(culof_context* ctx, void* cuda_stream) {
    return guarded([&] { engine_of(ctx).set_stream(static_cast<cudaStream_t>(cuda_stream)); });
}

int culof_context_synchronize(culof_context* ctx) {
    return guarded([&] { engine_of(ctx).check_status(); });
}

int culof_context_set_path(culof_context* ctx, int path) {
    return guarded([&] {
        if (path < CULOF_PATH_AUTO || path > CULOF_PATH_TENSOR)
            throw Error(culof_gb300::kInvalidArgument, "unknown path");
        engine_of(ctx).set_path(path);
    });
}

int culof_context_last_path(culof_context* ctx) {
    int p = -1;
    guarded([&] { p = engine_of(ctx).last_path(); });
    return p;
}

int culof_context_set_timing(culof_context* ctx, int on) {
    return guarded([&] { engine_of(ctx).set_timing(on != 0); });
}

int culof_context_stage_times(culof_context* ctx, float* ms, int cap) {
    return guarded([&] {
        if (ms == nullptr || cap < 0) throw Error(culof_gb300::kInvalidArgument, "ms must not be null");
        engine_of(ctx).stage_times(ms, cap);
    });
}

unsigned long long culof_kernel_launch_count(void) { return culof_gb300::launch_count(); }

int culof_context_pair_stats(culof_context* ctx, double* evaluated_pairs, double* total_pairs) {
    return guarded([&] { engine_of(ctx).pair_stats(evaluated_pairs, total_pairs); });
}

int culof_context_probe_bounded_wait(culof_context* ctx, long long spin_limit) {
    return guarded([&] { engine_of(ctx).probe_bounded_wait(spin_limit); });
}

int culof_lof(const float* points, int64_t n_points, int n_dims, int k, int normalize, float* scores_out) {
    return guarded([&] {
        culof_gb300::validate_lof_args(points, n_points, n_dims, k);
        require_device();
        thread_engine().lof_host(points, n_points, n_dims, k, normalize != 0, scores_out);
    });
}

int culof_context_lof(culof_context* ctx, const float* points, int64_t n_points, int n_dims, int k,
                      int normalize, float* scores_out) {
    return guarded([&] { engine_of(ctx).lof_host(points, n_points, n_dims, k, normalize != 0, scores_out); });
}

int culof_fit_predict(const float* points, int64_t n_points, int n_dims, int k, int normalize,
                      double contamination, float* nof_out, int64_t* labels_out, double* offset_out) {
    return guarded([&] {
        culof_gb300::validate_lof_args(points, n_points, n_dims, k);
        require_device();
        thread_engine().fit_predict_host(points, n_points, n_dims, k, normalize != 0, contamination, nof_out,
                                         labels_out, offset_out);
    });
}

int culof_context_fit_predict(culof_context* ctx, const float* points, int64_t n_points, int n_dims, int k,
                              int normalize, double contamination, float* nof_out, int64_t* labels_out,
                              double* offset_out) {
    return guarded([&] {
        engine_of(ctx).fit_predict_host(points, n_points, n_dims, k, normalize != 0, contamination, nof_out,
                                        labels_out, offset_out);
    });
}

int culof_context_lof_device(culof_context* ctx, const float* d_points, int64_t n_points, int n_dims, int k,
                             int normalize, float* d_scores) {
    return guarded([&] {
        if (d_scores == nullptr) throw Error(culof_gb300::kInvalidArgument, "d_scores must not be null");
        engine_of(ctx).lof_device(d_points, n_points, n_dims, k, normalize != 0, d_scores, nullptr);
    });
}

int culof_context_fit_predict_device(culof_context* ctx, const float* d_points, int64_t n_points, int n_dims,
                                     int k, int normalize, double contamination, float* d_nof,
                                     int64_t* d_labels, double* d_offset) {
    return guarded([&] {
        engine_of(ctx).fit_predict_device(d_points, n_points, n_dims, k, normalize != 0, contamination, d_nof,
                                          d_labels, d_offset);
    });
}

int culof_choose_tile_rows(int64_t n_points, size_t budget_bytes) {
    return culof_gb300::choose_tile_rows(n_points, budget_bytes);
}

int culof_select_knn_tile(void* cuda_stream, float* d_tile, const float* d_norms, int rows, int64_t row_offset,
                          int64_t n_points, int k, int32_t* d_nbr_idx, float* d_nbr_d2, float* d_kdist2) {
    return guarded([&] {
        if (!d_tile || !d_norms || !d_nbr_idx || !d_nbr_d2 || !d_kdist2)
            throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        if (rows < 0 || row_offset < 0 || row_offset + rows > n_points)
            throw Error(culof_gb300::kInvalidArgument, "rows out of range");
        if (k < 1 || k > n_points) throw Error(culof_gb300::kInvalidArgument, "k must satisfy 1 <= k <= n_points");
        culof_gb300::select_tile_rows(d_tile, d_norms, rows, row_offset, n_points, k, culof_gb300::kSelectGram,
                                       d_nbr_idx, d_nbr_d2, d_kdist2, static_cast<cudaStream_t>(cuda_stream));
    });
}

int culof_context_knn_device(culof_context* ctx, const float* d_points, int64_t n_points, int n_dims, int k,
                             int normalize, int32_t* d_nbr_idx, float* d_nbr_d2, float* d_kdist2) {
    return guarded([&] {
        if (!d_nbr_idx || !d_nbr_d2 || !d_kdist2)
            throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        engine_of(ctx).knn(d_points, n_points, n_dims, k, normalize != 0, d_nbr_idx, d_nbr_d2, d_kdist2);
    });
}

int culof_compute_lrd(void* cuda_stream, const int32_t* d_nbr_idx, const float* d_nbr_d2, const float* d_kdist2,
                      int64_t n_points, int k, float* d_lrd) {
    return guarded([&] {
        if (!d_nbr_idx || !d_nbr_d2 || !d_kdist2 || !d_lrd)
            throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        if (n_points < 1 || k < 1) throw Error(culof_gb300::kInvalidArgument, "n_points and k must be >= 1");
        culof_gb300::compute_lrd(d_nbr_idx, d_nbr_d2, d_kdist2, n_points, k, d_lrd, nullptr,
                                 static_cast<cudaStream_t>(cuda_stream));
    });
}

int culof_compute_scores(void* cuda_stream, const int32_t* d_nbr_idx, const float* d_lrd, int64_t n_points,
                         int k, float* d_scores) {
    return guarded([&] {
        if (!d_nbr_idx || !d_lrd || !d_scores)
            throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        if (n_points < 1 || k < 1) throw Error(culof_gb300::kInvalidArgument, "n_points and k must be >= 1");
        culof_gb300::compute_scores(d_nbr_idx, d_lrd, n_points, k, d_scores, nullptr, nullptr,
                                    static_cast<cudaStream_t>(cuda_stream));
    });
}

int culof_context_knn_shard_device(culof_context* ctx, const float* d_points, int64_t n_points, int n_dims, int k,
                                   int normalize, int shard, int num_shards, int32_t* d_nbr_idx, float* d_nbr_d2,
                                   float* d_kdist2, int32_t* d_rows, int64_t* rows_out) {
    return guarded([&] {
        if (!d_nbr_idx || !d_nbr_d2 || !d_kdist2 || !d_rows)
            throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        const int64_t m = engine_of(ctx).knn_shard(d_points, n_points, n_dims, k, normalize != 0, shard, num_shards,
                                                   d_nbr_idx, d_nbr_d2, d_kdist2, d_rows);
        if (rows_out) *rows_out = m;
    });
}

int culof_compute_lrd_rows(void* cuda_stream, const int32_t* d_nbr_idx, const float* d_nbr_d2,
                           const float* d_kdist2, int64_t n_points, int k, const int32_t* d_rows, int64_t num_rows,
                           float* d_lrd) {
    return guarded([&] {
        if (!d_nbr_idx || !d_nbr_d2 || !d_kdist2 || !d_lrd || !d_rows)
            throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        if (n_points < 1 || k < 1) throw Error(culof_gb300::kInvalidArgument, "n_points and k must be >= 1");
        if (num_rows < 0 || num_rows > n_points) throw Error(culof_gb300::kInvalidArgument, "num_rows out of range");
        culof_gb300::compute_lrd(d_nbr_idx, d_nbr_d2, d_kdist2, n_points, k, d_lrd, nullptr,
                                 static_cast<cudaStream_t>(cuda_stream), d_rows, num_rows);
    });
}

int culof_compute_scores_rows(void* cuda_stream, const int32_t* d_nbr_idx, const float* d_lrd, int64_t n_points,
                              int k, const int32_t* d_rows, int64_t num_rows, float* d_scores) {
    return guarded([&] {
        if (!d_nbr_idx || !d_lrd || !d_scores || !d_rows)
            throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        if (n_points < 1 || k < 1) throw Error(culof_gb300::kInvalidArgument, "n_points and k must be >= 1");
        if (num_rows < 0 || num_rows > n_points) throw Error(culof_gb300::kInvalidArgument, "num_rows out of range");
        culof_gb300::compute_scores(d_nbr_idx, d_lrd, n_points, k, d_scores, nullptr, nullptr,
                                    static_cast<cudaStream_t>(cuda_stream), d_rows, num_rows);
    });
}

int culof_context_bf16_gram(culof_context* ctx, const void* d_A, int64_t rows_a, const void* d_B, int64_t rows_b,
                            int K, float* d_G) {
    return guarded([&] {
        if (!d_A || !d_B || !d_G) throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        engine_of(ctx).bf16_gram(d_A, rows_a, d_B, rows_b, K, d_G);
    });
}

int culof_context_lof_batched_device(culof_context* ctx, int num_problems, const int64_t* offsets, const int* ks,
                                     const float* d_points, int n_dims, int normalize, float* d_scores) {
    return guarded([&] {
        engine_of(ctx).lof_batched_device(num_problems, offsets, ks, d_points, n_dims, normalize != 0, d_scores);
    });
}

int culof_lof_batched(int num_problems, const int64_t* offsets, const int* ks, const float* points, int n_dims,
                      int normalize, float* scores_out) {
    return guarded([&] {
        require_device();
        thread_engine().lof_batched_host(num_problems, offsets, ks, points, n_dims, normalize != 0, scores_out);
    });
}

int culof_context_lof_batched(culof_context* ctx, int num_problems, const int64_t* offsets, const int* ks,
                              const float* points, int n_dims, int normalize, float* scores_out) {
    return guarded([&] {
        engine_of(ctx).lof_batched_host(num_problems, offsets, ks, points, n_dims, normalize != 0, scores_out);
    });
}

int culof_context_set_graphs(culof_context* ctx, int on) {
    return guarded([&] { engine_of(ctx).set_graphs(on != 0); });
}

int culof_context_batched_tuning(culof_context* ctx, float* ms4, int* ctas_per_sm, int* pairs_per_lane) {
    return guarded([&] {
        if (!ms4 || !ctas_per_sm || !pairs_per_lane)
            throw Error(culof_gb300::kInvalidArgument, "output pointers must not be null");
        engine_of(ctx).batched_tuning(ms4, ctas_per_sm, pairs_per_lane);
    });
}

int culof_context_lof_backward_device(culof_context* ctx, const float* d_points, int64_t n_points, int n_dims, int k,
                                      int normalize, const int32_t* d_nbr_idx, const double* d_grad_scores,
                                      double* d_grad_points, double* d_scores_out) {
    return guarded([&] {
        engine_of(ctx).lof_backward_device(d_points, n_points, n_dims, k, normalize != 0, d_nbr_idx, d_grad_scores,
                                           d_grad_points, d_scores_out);
    });
}

int culof_context_contamination_offset_device(culof_context* ctx, const float* d_nof, int64_t n_points,
                                              double contamination, double* d_offset) {
    return guarded([&] {
        if (!d_nof || !d_offset) throw Error(culof_gb300::kInvalidArgument, "device pointers must not be null");
        if (n_points < 1) throw Error(culof_gb300::kInvalidArgument, "n_points must be >= 1");
        engine_of(ctx).offset_device(d_nof, n_points, contamination, d_offset);
    });
}

}  // extern "C"

// ---- C++ API (include/culof.h) ----------------------------------------------

namespace culof {

bool cuda_available() { return culof_cuda_available() != 0; }

std::string device_info() {
    char buf[512];
    if (culof_device_info(buf, sizeof buf) != CULOF_OK) return "unknown device";
    return buf;
}

std::vector<float> lof(const float* points, int n_points, int n_dims, int k, bool normalize) {
    std::vector<float> out(n_points > 0 ? static_cast<size_t>(n_points) : 0);
    const int rc = culof_lof(points, n_points, n_dims, k, normalize ? 1 : 0, out.data());
    if (rc == CULOF_ERR_INVALID_ARGUMENT) throw std::invalid_argument(culof_last_error());
    if (rc != CULOF_OK) throw CudaError(culof_last_error());
    return out;
}

}  // namespace culof
