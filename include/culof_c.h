/*
 * culof_gb300 C ABI: the drop-in boundary of the exact-LOF fit_predict path.
 *
 * Plain C: pointers, sizes and status codes, no C++ types, no exceptions, no
 * torch. Every entry point returns CULOF_OK (0) or an error status; the
 * message of the calling thread's last failure is culof_last_error().
 *
 * Each function names the reference interface it replaces (paths within the
 * Aminsed/cuLOF 0.2.0 source tree). Host-pointer entry points are synchronous
 * like the reference's culof::lof; *_device entry points take device pointers
 * and run asynchronously on the context's stream.
 *
 * Threads: a context must not be used by two threads at once. The entry
 * points without a context argument use a per-thread default context.
 */
#ifndef CULOF_C_H
#define CULOF_C_H

#include <stddef.h>
#include <stdint.h>

#if defined(__GNUC__)
#define CULOF_API __attribute__((visibility("default")))
#else
#define CULOF_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

#define CULOF_OK 0
#define CULOF_ERR_INVALID_ARGUMENT 1 /* culof::lof's std::invalid_argument (pipeline.cu:133-141) */
#define CULOF_ERR_CUDA 2             /* culof::CudaError (pipeline.cu:17-23)                     */
#define CULOF_ERR_NO_DEVICE 3        /* CudaError("no CUDA device available") (pipeline.cu:142)  */
#define CULOF_ERR_INTERNAL 4
#define CULOF_ERR_KERNEL 5 /* a kernel reported an error status word (e.g. a bounded wait expired) */

/* Path selection for culof_context_set_path. */
#define CULOF_PATH_AUTO 0    /* GENERAL for n <= 4096; FAST for d <= 8; TENSOR above; GENERAL past the fused limits */
#define CULOF_PATH_FAST 1    /* fused FP32 distance + filtered select (d <= 128, k <= 64) */
#define CULOF_PATH_GENERAL 2 /* exact distance tile + radix select (any d, any k)        */
#define CULOF_PATH_TENSOR 3  /* f16 tensor-core filter + exact rescoring (d <= 128, k <= 64) */

typedef struct culof_context culof_context;

/* Version string of the API this library implements: "0.2.0"
 * (src/culof/_version.py:8). */
CULOF_API const char* culof_version(void);

/* Message of the calling thread's last failed call ("" if none). */
CULOF_API const char* culof_last_error(void);

/* include/culof.h:28 culof::cuda_available(). 1 if a CUDA device is usable. */
CULOF_API int culof_cuda_available(void);

/* include/culof.h:31 culof::device_info(): "<name> (sm_XY, <SMs> SMs, <MiB> MiB)",
 * written NUL-terminated into buf (truncated to cap). */
CULOF_API int culof_device_info(char* buf, size_t cap);

/* Contexts own a stream and grow-only device workspaces, replacing the
 * reference's per-call Stream/Buffer objects (pipeline.cu:43-74, 148-168).
 * The context binds to the device current at creation. */
CULOF_API int culof_context_create(culof_context** out);
CULOF_API void culof_context_destroy(culof_context* ctx);
/* Run on a caller's cudaStream_t (NULL: the context's own stream). Part of a
 * call may run on two streams of the context forked from that stream by an
 * event and joined back to it before the call's later work: everything a
 * call writes is ordered on the call's stream as if it ran there alone. */
CULOF_API int culof_context_set_stream(culof_context* ctx, void* cuda_stream);
CULOF_API int culof_context_synchronize(culof_context* ctx);
/* CULOF_PATH_* (default AUTO). Every path returns bit-identical results. */
CULOF_API int culof_context_set_path(culof_context* ctx, int path);
/* Path used by the last k-NN run of this context (CULOF_PATH_FAST/GENERAL/TENSOR). */
CULOF_API int culof_context_last_path(culof_context* ctx);

/* include/culof.h:46-47 culof::lof(points, n, d, k, normalize).
 * points: host, row-major (n_points x n_dims) float32. scores_out: host,
 * n_points floats (positive LOF). Synchronous. */
CULOF_API int culof_lof(const float* points, int64_t n_points, int n_dims, int k, int normalize,
              float* scores_out);
CULOF_API int culof_context_lof(culof_context* ctx, const float* points, int64_t n_points, int n_dims, int k,
                      int normalize, float* scores_out);

/* src/culof/__init__.py:173-191 LOF(n_neighbors=k, contamination, normalize)
 * .fit(X) followed by predict(): negative_outlier_factor_ (= -lof), offset_
 * and the labels (-1 outlier, 1 inlier). contamination <= 0 means 'auto'
 * (offset_ = -1.5); otherwise it must be in (0, 0.5] and offset_ equals
 * np.percentile(nof, 100 * contamination) exactly. Host pointers; any
 * output may be NULL. Synchronous. */
CULOF_API int culof_fit_predict(const float* points, int64_t n_points, int n_dims, int k, int normalize,
                      double contamination, float* nof_out, int64_t* labels_out,
                      double* offset_out);
CULOF_API int culof_context_fit_predict(culof_context* ctx, const float* points, int64_t n_points, int n_dims,
                              int k, int normalize, double contamination, float* nof_out,
                              int64_t* labels_out, double* offset_out);

/* Device-resident forms of the two calls above (inputs already in HBM):
 * every pointer is device memory; work is queued on the context stream and
 * the call returns without synchronising. */
CULOF_API int culof_context_lof_device(culof_context* ctx, const float* d_points, int64_t n_points, int n_dims,
                             int k, int normalize, float* d_scores);
CULOF_API int culof_context_fit_predict_device(culof_context* ctx, const float* d_points, int64_t n_points,
                                     int n_dims, int k, int normalize, double contamination,
                                     float* d_nof, int64_t* d_labels, double* d_offset);

/* Per-stage timing with CUDA events on the context stream (off by default).
 * culof_context_stage_times writes milliseconds of the last call for up to
 * cap stages (0 centre+norms, 1 spatial order+tiles, 2 seed, 3 sweep or tile
 * select, 4 merge, 5 lrd+score, 6 offset+labels; -1 = did not run) and
 * synchronises the stream. No reference counterpart: measurement support. */
CULOF_API int culof_context_set_timing(culof_context* ctx, int on);
CULOF_API int culof_context_stage_times(culof_context* ctx, float* ms, int cap);

/* Kernels launched by this library in this process so far. No reference
 * counterpart: measurement support. */
CULOF_API unsigned long long culof_kernel_launch_count(void);
/* Row x column pairs the last small-d FP32 sweep of this context evaluated
 * (tiles that a bounding-box test proves farther than every k-th neighbour
 * are skipped) and the pairs it would evaluate without that test (every
 * column tile past the seed's own and four neighbour tiles); both 0 after
 * other paths. Synchronises the context stream. */
CULOF_API int culof_context_pair_stats(culof_context* ctx, double* evaluated_pairs, double* total_pairs);

/* Test support for the failure path. Every wait in the library's kernels is
 * bounded: when it runs out, the kernel sets the context's status word and
 * returns, and the call fails with CULOF_ERR_KERNEL while the context stays
 * usable. This runs one such wait on a barrier phase that nothing completes,
 * giving up after spin_limit polls (1 .. 2^24), so it returns
 * CULOF_ERR_KERNEL. Synchronises the context stream. */
CULOF_API int culof_context_probe_bounded_wait(culof_context* ctx, long long spin_limit);

/* Measured FP32 CUDA-core throughput of the current device in TFLOP/s
 * (packed = 1: fma.rn.f32x2; 0: scalar fma.rn.f32), the roofline
 * denominator of the FP32 distance sweep. No reference counterpart. */
CULOF_API int culof_probe_fp32_tflops(int packed, double* tflops_out);

/* ---- stage entry points (the reference's internal stage API) ---------- */

/* include/culof_internal.cuh:63 choose_tile_rows (pipeline.cu:33-38):
 * clamp(budget_bytes / (4 n_points), 1, n_points). */
CULOF_API int culof_choose_tile_rows(int64_t n_points, size_t budget_bytes);

/* include/culof_internal.cuh:52-53 select_knn (knn.cu:119-241), same tile
 * contract: d_tile holds rows x n_points Gram values x_(row_offset+r).x_c,
 * converted in place to max(0, |x_r|^2 + |x_c|^2 - 2 x_r.x_c) with +inf on
 * the diagonal; emits the k neighbours of each row in transposed layout
 * (slot t of point i at [t * n_points + i]) and the k-th squared distance.
 * Bit-exact with the reference's kernel for identical tile and norms. */
CULOF_API int culof_select_knn_tile(void* cuda_stream, float* d_tile, const float* d_norms, int rows,
                          int64_t row_offset, int64_t n_points, int k, int32_t* d_nbr_idx,
                          float* d_nbr_d2, float* d_kdist2);

/* The exact k-NN stage of culof::lof (pipeline.cu:162-195: centre, norms,
 * distance tiles, select) with exact float32 direct-difference distances.
 * d_points device (n x d); outputs device, transposed (k x n) + kdist2 (n). */
CULOF_API int culof_context_knn_device(culof_context* ctx, const float* d_points, int64_t n_points, int n_dims,
                             int k, int normalize, int32_t* d_nbr_idx, float* d_nbr_d2,
                             float* d_kdist2);

/* ---- row-sharded run (one rank per GPU; the multi-GPU plan) -----------
 * The reference splits its k-NN stage into row tiles on one GPU
 * (pipeline.cu:175-195); these entry points split it into shards across
 * ranks. Each rank holds all n points and computes its shard's neighbours
 * against all of them with no communication; the LOF then needs two
 * exchanges of n floats: the k-distances before the LRD and the LRDs before
 * the scores. Every entry is written by exactly one shard, so the exchange
 * can be an all-reduce (sum) of zero-initialised n-float arrays, exact.
 *
 * culof_context_knn_shard_device: shard `shard` of num_shards (0 <= shard <
 * num_shards) of culof_context_knn_device. The fused paths shard blocks of
 * the engine's spatial order (row tiles of 128 points, the same order on
 * every rank for the same points); the general path shards blocks of
 * original rows. Outputs, device, written only at the shard's rows: slot t
 * of point i at [t * n_points + i] of d_nbr_idx / d_nbr_d2 and d_kdist2[i];
 * d_rows (n_points capacity) receives the shard's original row indices and
 * *rows_out (host, nullable) their count. The shards of one problem list
 * disjoint rows that cover all n, and each row's results are bit-identical
 * to the unsharded call's. Asynchronous on the context stream. */
CULOF_API int culof_context_knn_shard_device(culof_context* ctx, const float* d_points, int64_t n_points, int n_dims,
                                             int k, int normalize, int shard, int num_shards, int32_t* d_nbr_idx,
                                             float* d_nbr_d2, float* d_kdist2, int32_t* d_rows, int64_t* rows_out);

/* include/culof_internal.cuh:56-58 compute_lrd (lof.cu:32-46) for a row
 * block: the LRD of the num_rows points d_rows lists (d_lrd[i] for each
 * listed i), given the (k x n) slots of those points and all n k-distances. */
CULOF_API int culof_compute_lrd_rows(void* cuda_stream, const int32_t* d_nbr_idx, const float* d_nbr_d2,
                                     const float* d_kdist2, int64_t n_points, int k, const int32_t* d_rows,
                                     int64_t num_rows, float* d_lrd);

/* include/culof_internal.cuh:60-62 compute_scores (lof.cu:49-62) for a row
 * block: d_scores[i] for each listed i, given all n LRDs. */
CULOF_API int culof_compute_scores_rows(void* cuda_stream, const int32_t* d_nbr_idx, const float* d_lrd,
                                        int64_t n_points, int k, const int32_t* d_rows, int64_t num_rows,
                                        float* d_scores);

/* include/culof_internal.cuh:56-58 compute_lrd (lof.cu:32-46). Device pointers. */
CULOF_API int culof_compute_lrd(void* cuda_stream, const int32_t* d_nbr_idx, const float* d_nbr_d2,
                      const float* d_kdist2, int64_t n_points, int k, float* d_lrd);

/* include/culof_internal.cuh:60-62 compute_scores (lof.cu:49-62). Device pointers. */
CULOF_API int culof_compute_scores(void* cuda_stream, const int32_t* d_nbr_idx, const float* d_lrd,
                         int64_t n_points, int k, float* d_scores);

/* Batched LOF (no reference counterpart: the reference serves one problem
 * per culof::lof call, pipeline.cu:131-207). Positive LOF scores of
 * num_problems independent problems in one call: d_points holds every
 * problem's points concatenated (row-major float32, n_dims columns, device),
 * offsets (host, num_problems + 1 entries, offsets[0] = 0) delimits them and
 * ks (host) gives each problem's k; d_scores (device, offsets[num_problems]
 * floats) receives the scores in the same order. Each problem obeys the
 * reference's rules (n >= 2, 1 <= k < n) and the batched limits k <= 48,
 * n_dims <= 64. Every problem's scores are bit-identical to a single-problem
 * culof_context_lof call. The first call with a batch layout plans it and
 * times the kernel variants; the launch sequence is then captured as a CUDA
 * graph and replayed while the layout, the two pointers and the stream stay
 * the same. Asynchronous on the context stream. */
CULOF_API int culof_context_lof_batched_device(culof_context* ctx, int num_problems, const int64_t* offsets,
                                               const int* ks, const float* d_points, int n_dims, int normalize,
                                               float* d_scores);
/* The same on host arrays: copies in, runs, copies out, synchronises
 * (points and scores_out host, offsets and ks as above). */
CULOF_API int culof_lof_batched(int num_problems, const int64_t* offsets, const int* ks, const float* points,
                                int n_dims, int normalize, float* scores_out);
CULOF_API int culof_context_lof_batched(culof_context* ctx, int num_problems, const int64_t* offsets, const int* ks,
                                        const float* points, int n_dims, int normalize, float* scores_out);
/* Graph capture of repeated batched calls: on (1, default) or off (0). */
CULOF_API int culof_context_set_graphs(culof_context* ctx, int on);
/* The batched autotuner's record for the context's current batch layout
 * (measurement support; no reference counterpart): ms4[2 (c - 1) + (p - 1)]
 * is the whole batched call's time in milliseconds with the k-NN kernel at
 * c CTAs per SM and p column pairs per lane (-1 if that variant was not
 * tried: two CTAs need the shared memory, two pairs d <= 16), and *ctas_per_sm /
 * *pairs_per_lane the chosen variant (0 before the first batched call). */
CULOF_API int culof_context_batched_tuning(culof_context* ctx, float* ms4, int* ctas_per_sm, int* pairs_per_lane);

/* Sparse LOF backward (no reference counterpart: the reference has no
 * gradient). Gradient of L = sum_i g_i score_i with respect to the points, the
 * neighbour sets held fixed: d_nbr_idx is the k x n slot array of a forward
 * k-NN of the same points (culof_context_knn_device; slot k-1 designates the
 * k-th neighbour), d_grad_scores n doubles (g), d_grad_points n x d doubles
 * (row-major, written), d_scores_out n doubles (nullable: the FP64 scores of
 * the same fixed-neighbour forward). Evaluated in FP64, deterministic (no
 * floating-point atomics). Requires n_points * k < 2^31. Asynchronous on the
 * context stream; a neighbour index out of range surfaces as CULOF_ERR_KERNEL
 * at culof_context_synchronize. */
CULOF_API int culof_context_lof_backward_device(culof_context* ctx, const float* d_points, int64_t n_points,
                                                int n_dims, int k, int normalize, const int32_t* d_nbr_idx,
                                                const double* d_grad_scores, double* d_grad_points,
                                                double* d_scores_out);

/* The tensor-core building block of the precision form: G = A B^T for
 * row-major bf16 operands A (rows_a x K) and B (rows_b x K), f32 accumulation
 * (tcgen05.mma, TMEM). rows_a and rows_b multiples of 128, K = 128; device
 * pointers 16-byte aligned; G row-major (rows_a x rows_b). Asynchronous on the
 * context stream; errors surface at culof_context_synchronize. No reference
 * counterpart (the reference's Gram tile is cuBLAS SGEMM, pipeline.cu:182-188). */
CULOF_API int culof_context_bf16_gram(culof_context* ctx, const void* d_A, int64_t rows_a, const void* d_B,
                                      int64_t rows_b, int K, float* d_G);

/* src/culof/__init__.py:179-185 offset_: np.percentile(d_nof, 100 * contamination)
 * computed on the GPU (contamination <= 0: 'auto', -1.5). d_offset: device double. */
CULOF_API int culof_context_contamination_offset_device(culof_context* ctx, const float* d_nof,
                                              int64_t n_points, double contamination,
                                              double* d_offset);

/* The same offset as culof_context_contamination_offset_device, for callers
 * that cannot allocate device memory while they run (an operator inside a
 * framework that owns all device memory through its own pool, a loop that
 * must not stall on cudaMalloc/cudaFree). It allocates nothing: the caller
 * passes device buffers for d_nof and d_offset, and the select's scratch is a
 * fixed 8,232-byte array in this library's device memory, which every GPU
 * that loads the library holds until the process exits. n_points must be at
 * most 2^31 - 1 (larger sizes are rejected with CULOF_ERR_INVALID_ARGUMENT).
 * The first call on a device looks up the array's address (cudaGetSymbolAddress);
 * make it before any stream capture. The address is cached per device and
 * CUDA context, so a re-created context (cudaDeviceReset) gets its own
 * lookup on its first call. Every call shares the array and clears it first;
 * calls that overlap on the GPU race on it. Asynchronous on cuda_stream,
 * which must belong to the current device. It has no counterpart in the
 * reference. */
CULOF_API int culof_contamination_offset_noalloc(void* cuda_stream, const float* d_nof, int64_t n_points,
                                                 double contamination, double* d_offset);

#ifdef __cplusplus
}
#endif

#endif /* CULOF_C_H */
