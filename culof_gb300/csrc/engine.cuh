// The engine behind a culof_context: stream, device workspaces, pipeline.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "common.cuh"
#include "prep.cuh"

namespace culof_gb300 {

// Grow-only device allocation. Replaces the reference's per-call Buffer RAII
// objects (pipeline.cu:43-59): a context keeps its workspaces between calls.
class DevBuf {
public:
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() { release(); }
    void* get(size_t bytes);
    template <typename T>
    T* as(size_t count) {
        return static_cast<T*>(get(count * sizeof(T)));
    }
    void release();
    size_t capacity() const { return cap_; }

private:
    void* ptr_ = nullptr;
    size_t cap_ = 0;
};

// A batch of independent problems (batched.cu): host plan and device copies.
struct BatchPlan {
    int num = 0;
    int d = 0;
    bool normalize = false;
    std::vector<int64_t> off, nkoff, coff, toff;  // points, k-NN slots, centring chunks, row tiles (prefix sums)
    std::vector<int> ks;
    std::vector<uint2> items;  // (problem, row tile), largest problems first
    int64_t ntot = 0, nchunks = 0;
};
struct BatchDev {
    int64_t *off = nullptr, *nkoff = nullptr, *coff = nullptr;
    int* ks = nullptr;
    uint2* items = nullptr;
    int* cp = nullptr;  // problem of each centring chunk
    int nitems = 0, d = 0;
    int* pid = nullptr;  // problem of each point
    float* xc = nullptr;
    double *partial = nullptr, *mean = nullptr, *inv = nullptr;
    int32_t* nbr = nullptr;
    float *d2 = nullptr, *kd = nullptr, *lrd = nullptr;
    unsigned* counter = nullptr;
    // spatial order: sorted coordinates, original index of each sorted point
    float* xs = nullptr;
    unsigned* lidx = nullptr;
    float* pmm = nullptr;
    int* pdims = nullptr;
    unsigned *skeys = nullptr, *svals = nullptr, *scounts = nullptr;
    // tiles of 128 sorted points: problem, first tile per problem, boxes
    int* tpid = nullptr;
    int64_t* toff = nullptr;
    int64_t ntiles = 0;
    float* tbox = nullptr;
};

enum Path : int { kPathAuto = 0, kPathFast = 1, kPathGeneral = 2, kPathTensor = 3 };

class Engine {
public:
    explicit Engine(int device);
    ~Engine();
    Engine(const Engine&) = delete;
    Engine& operator=(const Engine&) = delete;

    int device() const { return device_; }
    cudaStream_t stream() const { return stream_; }
    void set_stream(cudaStream_t s) { stream_ = s ? s : own_stream_; }
    void set_path(int p) { path_ = p; }
    int last_path() const { return last_path_; }

    // Centre (+ z-score), norms and exact k-NN; outputs device, transposed.
    void knn(const float* d_x, int64_t n, int d, int k, bool normalize, int32_t* nbr_idx,
             float* nbr_d2, float* kdist2);
    // One shard of a row-sharded k-NN: the neighbours of the shard's rows
    // against all n points, written at the rows' own columns of the (k x n)
    // outputs; rows (n capacity) receives the shard's original row indices.
    // Returns their count. Shards of the fused paths are blocks of the
    // spatial order's row tiles; the general path's are blocks of original
    // rows. Every row's results equal the unsharded call's.
    int64_t knn_shard(const float* d_x, int64_t n, int d, int k, bool normalize, int shard, int num_shards,
                      int32_t* nbr_idx, float* nbr_d2, float* kdist2, int32_t* rows);
    // Positive LOF scores (and optionally nof = -scores) on the device.
    void lof_device(const float* d_x, int64_t n, int d, int k, bool normalize, float* d_scores,
                    float* d_nof);
    // LOF.fit + predict on the device; d_offset is a device double.
    void fit_predict_device(const float* d_x, int64_t n, int d, int k, bool normalize,
                            double contamination, float* d_nof, int64_t* d_labels, double* d_offset);
    void offset_device(const float* d_nof, int64_t n, double contamination, double* d_offset);
    void bf16_gram(const void* A, int64_t rows_a, const void* B, int64_t rows_b, int K, float* G);
    // Gradient of sum_i g_i score_i with respect to the points (FP64), the
    // neighbour sets of a forward k-NN (nbr_idx, k x n) held fixed; optional
    // FP64 scores of the same fixed-neighbour forward.
    // LOF scores of many independent problems (points concatenated; host
    // offsets[num + 1], ks[num]) in one persistent launch, replayed from a
    // CUDA graph while the batch layout and pointers repeat.
    void lof_batched_device(int num, const int64_t* offsets, const int* ks, const float* d_x, int d, bool normalize,
                            float* d_scores);
    void lof_batched_host(int num, const int64_t* offsets, const int* ks, const float* x, int d, bool normalize,
                          float* scores);
    void set_graphs(bool on) { use_graphs_ = on; }
    // The batched autotuner's measurements for the current layout (times of
    // the whole batched call): ms4[2 (c - 1) + (p - 1)] for the k-NN kernel at
    // c CTAs per SM and p column pairs per lane (-1: not tried), and its
    // choice (0 before the first batched call).
    void batched_tuning(float* ms4, int* per_sm, int* pairs_per_lane) const;
    // Pairs the last FP32 small-d sweep evaluated and the pairs of an
    // unpruned sweep (both 0 for other paths); synchronises.
    void pair_stats(double* evaluated, double* total);
    void lof_backward_device(const float* d_x, int64_t n, int d, int k, bool normalize, const int32_t* nbr_idx,
                             const double* grad_scores, double* grad_x, double* scores_out);

    // Host-pointer forms: copy in, run, copy out, synchronise.
    void lof_host(const float* x, int64_t n, int d, int k, bool normalize, float* scores);
    void fit_predict_host(const float* x, int64_t n, int d, int k, bool normalize,
                          double contamination, float* nof, int64_t* labels, double* offset);

private:
    void batch_plan(int num, const int64_t* offsets, const int* ks, int d, bool normalize);
    bool batch_same_plan(int num, const int64_t* offsets, const int* ks, int d, bool normalize) const;
    void batch_launch(const float* d_x, float* d_scores);
    void batch_autotune(const float* d_x, float* d_scores);
    int choose_path(int64_t n, int d, int k) const;
    void knn_general(const float* xc, const float* norms, int64_t n, int d, int k, int32_t* nbr_idx,
                     float* nbr_d2, float* kdist2, int64_t row_begin, int64_t row_end);
    void knn_fast(const float* xc, const float* norms, int64_t n, int d, int k, bool tensor, int32_t* nbr_idx,
                  float* nbr_d2, float* kdist2, int shard = 0, int num_shards = 1, int32_t* shard_rows = nullptr);
    int64_t knn_core(const float* d_x, int64_t n, int d, int k, bool normalize, int shard, int num_shards,
                     int32_t* nbr_idx, float* nbr_d2, float* kdist2, int32_t* rows);
    int tile_rows_for(int64_t n);

    int device_;
    cudaStream_t own_stream_ = nullptr;
    cudaStream_t stream_ = nullptr;
    // Two streams forked from the call's stream for work that runs side by
    // side (the small-d sweep on the high one, the isolated rows' pass on
    // the side one), with the events that fork them and join them back;
    // created on first use.
    cudaStream_t high_stream_ = nullptr, side_stream_ = nullptr;
    cudaEvent_t fork_ev_ = nullptr, high_join_ = nullptr, side_join_ = nullptr;
    void make_fork_streams();
    int path_ = kPathAuto;
    int last_path_ = kPathAuto;

    DevBuf x_, xc_, partial_, mean_, inv_std_, norms_, max_norm_;
    DevBuf nbr_idx_, nbr_d2_, kdist2_, lrd_, scores_, nof_, labels_, offset_, offset_scratch_;
    DevBuf tile_, bw_;
    // batched path (batched.cu)
    BatchPlan bplan_;
    BatchDev bdev_;
    DevBuf bplan_off_, bplan_nkoff_, bplan_coff_, bplan_ks_, bplan_items_, bplan_cp_;
    DevBuf bpid_, bxc_, bpartial_, bmean_, binv_, bnbr_, bd2_, bkd_, blrd_, bcounter_;
    DevBuf bxs_, blidx_, bpmm_, bpdims_, bskeys_, bsvals_, bscounts_;
    DevBuf bplan_toff_, bplan_tpid_, btbox_;
    bool use_graphs_ = true;
    bool btuned_ = false, btune_packed_ = true, bbest_packed_ = true;
    int btune_grid_ = 152, bbest_grid_ = 152;
    float btune_ms_[4] = {-1.0f, -1.0f, -1.0f, -1.0f};  // (CTAs per SM 1..2) x (column pairs 1..2)
    cudaGraphExec_t bgraph_exec_ = nullptr;
    bool bgraph_valid_ = false;
    const float* bgraph_x_ = nullptr;
    float* bgraph_scores_ = nullptr;
    cudaStream_t bgraph_stream_ = nullptr;
    unsigned long long bgraph_kernels_ = 0;
    // fast path workspaces
    DevBuf morton_, perm_, sort_tmp_, sort_hist_, cols_, rows_, tc_lists_, tiles_;
    // the FP32 sweep's evaluated (warp x column tile) blocks; the total it
    // would evaluate without pruning
    DevBuf pair_stats_, boxes_, plist_, pcount_, order_;
    // isolated rows of the small-d sweep: threshold, count, list and flags;
    // dimension-major columns and quarter-tile boxes
    DevBuf iso_, iso_cols_;
    unsigned long long stat_total_blocks_ = 0;
    // Device status word of the current call: kernels set it (a bounded wait
    // that expired, an out-of-range neighbour index); host paths check it.
    DevBuf status_;
    int* status_ptr() { return status_.as<int>(1); }

public:
    // Raises kKernelFault if a kernel of the last call reported an error
    // (synchronises the stream).
    void check_status();
    // Runs a bounded wait that never completes (limit polls) and reports it
    // like a kernel's expired wait: raises kKernelFault. Test support.
    void probe_bounded_wait(long long limit);

    // Stage timing with CUDA events on the launching stream. Stages:
    // 0 centre+norms, 1 spatial order+tiles, 2 seed, 3 sweep (or the general
    // path's tile+select), 4 merge, 5 lrd+score, 6 offset+labels.
    static constexpr int kNumStages = 7;
    void set_timing(bool on);
    // Milliseconds per stage of the last call (synchronises); -1 if a stage
    // did not run.
    void stage_times(float* ms, int cap);
    void mark(int boundary);

private:
    bool timing_ = false;
    cudaEvent_t events_[kNumStages + 1] = {};
    bool marked_[kNumStages + 1] = {};
};

unsigned long long launch_count();

// Argument validation shared by every entry point (pipeline.cu:133-141).
void validate_lof_args(const void* points, int64_t n, int d, int k);
void validate_contamination(double c);

}  // namespace culof_gb300
