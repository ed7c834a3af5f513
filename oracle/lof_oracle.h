/*
 * CPU oracle for exact Local Outlier Factor: TEST INFRASTRUCTURE ONLY.
 *
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load
 * this library, and only as the checker or as the timed CPU baseline. The
 * product (culof_gb300 / libculof_gb300.so) never links, loads or calls it.
 *
 * It restates, in plain C, the algorithm of the reference cuLOF 0.2.0 hot
 * path with the numeric choices this project pins down (every function cites
 * the reference file:line it follows):
 *
 *   centre (+ optional z-score)   src/cuda/preprocess.cu:31-72
 *   squared row norms             src/cuda/preprocess.cu:75-84
 *   exact k-NN select + tie rule  src/cuda/knn.cu:119-232
 *   local reachability density    src/cuda/lof.cu:32-46
 *   LOF score                     src/cuda/lof.cu:49-62
 *   contamination offset          src/culof/__init__.py:179-185 (np.percentile)
 *   labels                        src/culof/__init__.py:208-210
 *
 * Distances are squared Euclidean in float32, accumulated by direct
 * differences in a fixed order (t = a_f - b_f; s = fma(t, t, s), f ascending),
 * which the GPU engine reproduces bit for bit. The reference's own form
 * (|a|^2 + |b|^2 - 2 a.b over a cuBLAS Gram tile) is restated separately in
 * oracle_ref_select_tile() for the select-only bit-exactness check.
 *
 * Parity pinning: tests/golden/ holds scikit-learn LocalOutlierFactor outputs
 * (the reference's own test oracle, tests/python/conftest.py:10-12) and the
 * outputs of the reference's Python layer (offset_, labels) generated by
 * tests/golden/make_golden.py; tests/test_oracle_golden.py checks this oracle
 * against them.
 */
#ifndef LOF_ORACLE_H
#define LOF_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Rows per partial sum in the centring reduction (both the oracle and the GPU
 * kernels use this order, so the FP64 means agree bit for bit). */
#define ORACLE_CENTER_CHUNK 256

/* Centre each feature (and scale to unit variance when normalize != 0).
 * preprocess.cu:31-72. mean/inv_std may be NULL. */
void oracle_center(const float* x, int64_t n, int d, int normalize, float* xc,
                   double* mean, double* inv_std);

/* norms[i] = (float) sum_f (double) xc[i,f]^2.  preprocess.cu:75-84. */
void oracle_norms(const float* xc, int64_t n, int d, float* norms);

/* Squared distance by direct differences, float32, fixed order. */
float oracle_dist2(const float* a, const float* b, int d);

/* Exact k-NN of rows [row_begin, row_end) against all n rows of xc.
 * Outputs use the reference's transposed layout: entry t of point i at
 * [t * n + i] (culof_internal.cuh:48-50). Selection key is (d2 bits, index);
 * the k-distance is the k-th key's d2 (knn.cu:180-184); slot order is every
 * neighbour with d2 < kdist2 by ascending index, then the ties == kdist2 by
 * ascending index (knn.cu:190-224). Parallel over rows with nthreads threads
 * (<= 0: all online CPUs). */
void oracle_knn_rows(const float* xc, int64_t n, int d, int k, int64_t row_begin,
                     int64_t row_end, int32_t* nbr_idx, float* nbr_d2, float* kdist2,
                     int nthreads);

/* lrd[i] = (float)(1 / (sum_t sqrt((double) max(kdist2[j], d2_it)) / k + 1e-10)).
 * lof.cu:32-46, summed in slot order. */
void oracle_lrd(const int32_t* nbr_idx, const float* nbr_d2, const float* kdist2,
                int64_t n, int k, float* lrd);

/* scores[i] = (float)(sum_t (double) lrd[j] / (double) lrd[i] / k).  lof.cu:49-62. */
void oracle_score(const int32_t* nbr_idx, const float* lrd, int64_t n, int k,
                  float* scores);

/* Whole pipeline, lof(X, k, normalize) -> scores (positive LOF).
 * pipeline.cu:131-207. Returns 0, or -1 for invalid arguments. */
int oracle_lof(const float* x, int64_t n, int d, int k, int normalize, float* scores,
               int nthreads);

/* np.percentile(nof, 100 * contamination) for a float32 array nof, as the
 * reference's LOF.fit computes offset_ (__init__.py:183), returned exactly
 * (the float32 result widened to double). Sorts a private copy. */
double oracle_percentile_offset(const float* nof, int64_t n, double contamination);

/* labels[i] = nof[i] < (float) offset ? -1 : 1 (__init__.py:208-210). */
void oracle_labels(const float* nof, int64_t n, double offset, int64_t* labels);

/* Restatement of the reference's select over a Gram tile (knn.cu:119-232):
 * raw = (norms[self] + norms[j]) - 2 * tile[r, j]; d2 = +inf for the
 * diagonal and NaN, else max(0, raw); k-th smallest key; slots as above. */
void oracle_ref_select_tile(const float* tile, const float* norms, int rows,
                            int64_t row_offset, int64_t n, int k, int32_t* nbr_idx,
                            float* nbr_d2, float* kdist2);

/* oracle_knn_rows for an arbitrary list of m rows: rows[r]'s neighbours go
 * to column r of the (k x m) outputs (slot t at [t * m + r]) and its
 * k-distance to kdist2[r]. */
void oracle_knn_list(const float* xc, int64_t n, int d, int k, const int64_t* rows, int64_t m,
                     int32_t* nbr_idx, float* nbr_d2, float* kdist2, int nthreads);

/* FP64 brute force from the definitions (Breunig et al. 2000), as the
 * reference's cpu_lof (tests/cpp/test_culof.cu:39-80) computes them: the
 * yardstick of the float32 engine's error, not a bit-exact restatement.
 * oracle_knn_f64: the kk nearest of the m points rows[] (rows NULL: every
 * point, m ignored) by (Euclidean distance, index), row-major (m x kk),
 * ascending. oracle_lof_f64: the LOF scores. Both centre (and z-score) in
 * double first. */
void oracle_knn_f64(const float* x, int64_t n, int d, int normalize, int kk, const int64_t* rows,
                    int64_t m, int64_t* idx, double* dist, int nthreads);
int oracle_lof_f64(const float* x, int64_t n, int d, int k, int normalize, double* scores,
                   int nthreads);

#ifdef __cplusplus
}
#endif

#endif /* LOF_ORACLE_H */
