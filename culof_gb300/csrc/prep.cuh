// Stage interfaces shared between translation units (not part of the C ABI).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace culof_gb300 {

// ---- prep.cu -------------------------------------------------------------
size_t center_partial_count(int64_t n, int d);
void center(const float* x, int64_t n, int d, bool normalize, float* xc, double* partial,
            double* mean, double* inv_std, cudaStream_t s);
void squared_norms(const float* xc, int64_t n, int d, float* norms, unsigned int* max_norm_bits,
                   cudaStream_t s);

// ---- select.cu (general path: exact-distance tile + per-row select) -------
enum SelectMode : int {
    kSelectDistances = 0,  // tile holds exact squared distances; self is skipped
    kSelectGram = 1,       // tile holds Gram values (reference contract, knn.cu:136-156)
};
void distance_tile(const float* xc, int64_t n, int d, int64_t row0, int rows, float* tile,
                   cudaStream_t s);
void select_tile_rows(float* tile, const float* norms, int rows, int64_t row_offset, int64_t n, int k, int mode,
                      int32_t* nbr_idx, float* nbr_d2, float* kdist2, cudaStream_t s);
int choose_tile_rows(int64_t n_points, size_t budget_bytes);
// rows[i] = first + i for i < m.
void iota_rows(int32_t* rows, int64_t first, int64_t m, cudaStream_t s);

// ---- lof.cu ----------------------------------------------------------------
// status (may be null): the gathers return early when it is non-zero and set
// it to 2 if a neighbour index is out of range. rows (nullable): only the m
// listed points (a row block of a sharded run) are computed.
void compute_lrd(const int32_t* nbr_idx, const float* nbr_d2, const float* kdist2, int64_t n, int k,
                 float* lrd, int* status, cudaStream_t s, const int32_t* rows = nullptr, int64_t m = 0);
void compute_scores(const int32_t* nbr_idx, const float* lrd, int64_t n, int k, float* scores,
                    float* nof, int* status, cudaStream_t s, const int32_t* rows = nullptr, int64_t m = 0);

struct OffsetPlan {
    int64_t lo;          // lower order statistic (0-based, ascending nof)
    int use_upper;       // gamma >= 0.5: r = b - diff * w, else a + diff * w
    float w;             // (float) gamma or (float) (1 - gamma)
    int is_auto;         // contamination 'auto': offset = -1.5
};
OffsetPlan plan_offset(int64_t n, double contamination);

// Scratch for the offset select: histogram bins plus a small state block.
constexpr int kOffsetHistBins = 2048;
struct OffsetState {
    unsigned int prefix;   // key bits fixed so far
    int below;             // keys strictly below the prefix range
    unsigned int a_key;    // order statistic lo
    unsigned int min_gt;   // smallest key above a_key
    int count_le;          // keys <= a_key
    int pad;
    double offset;         // result, float32 value widened
    float offset_f;
    int pad2;
};
size_t offset_scratch_bytes();
void contamination_offset(const float* nof, int64_t n, const OffsetPlan& plan, void* scratch,
                          double* offset_out_dev, cudaStream_t s);
void labels_from_offset(const float* nof, int64_t n, const double* offset_dev, int64_t* labels,
                        cudaStream_t s);

}  // namespace culof_gb300
