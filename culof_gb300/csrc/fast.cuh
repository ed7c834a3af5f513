// Fused distance + filtered exact select (the fast k-NN path).
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace culof_gb300 {

// True when the fast path handles (n, d, k).
bool fast_path_supported(int64_t n, int d, int k);

// The wide-point variant (8 < d <= 128), wide.cu.
int wide_dims_padded(int d);
size_t wide_tiles_floats(int d, int nt);
void wide_build_tiles(const float* xc, const float* norms, int64_t n, int d, const unsigned* perm, int nt,
                      float* tiles, cudaStream_t s);
// Row tiles [t0, t0 + mt) of the nt (every call covers a block of row tiles;
// the whole problem is t0 = 0, mt = nt).
void wide_seed(const float* tiles, int nt, int t0, int mt, int d, int k, uint64_t* seed_keys,
               unsigned long long* kth_shared, cudaStream_t s);
void wide_sweep(const float* tiles, int nt, int t0, int mt, int nsplit, int d, int k, const unsigned* maxn,
                unsigned long long* kth_shared, uint64_t* partial, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs on the low key_bits bits of the
// keys (8 bits per pass); keys_tmp / vals_tmp are scratch of n entries and
// counts holds sort_pairs_counts(n) entries. Returns the buffer holding the
// sorted keys (keys or keys_tmp) and sets *vals_out to the sorted values.
size_t sort_pairs_counts(int64_t n);
unsigned* sort_pairs_stable(unsigned* keys, unsigned* vals, unsigned* keys_tmp, unsigned* vals_tmp, int64_t n,
                            int key_bits, unsigned* counts, cudaStream_t s, unsigned** vals_out);
// In-place exclusive prefix sum (one block; for index-sized arrays).
void exclusive_scan_u32(unsigned* data, int64_t len, cudaStream_t s);

// Shared by the FP32 and tensor-core sweeps (fast.cu).
int choose_splits(int nt, int sms);
// Merges the rows at sorted positions [pos0, pos1).
void launch_merge(const uint64_t* seed_keys, const uint64_t* partial, const unsigned* perm, int64_t n, int nt,
                  int64_t pos0, int64_t pos1, int nsplit, int k, int32_t* idx, float* d2, float* kd, cudaStream_t s);

// The tensor-core variant (tc_sweep.cu). Sorted-order arrays of one call:
// xh f16 operand rows [padded][Kp], xr FP32 coordinates [padded][dr], cn
// norms, ix original indices, scale a device record of the f16 scaling.
// split: each coordinate x (scaled) is carried as two f16 values, hi =
// f16(x) and lo = f16(x - hi); the row operand holds [hi, lo, hi] and the
// column operand [hi, hi, lo] (d values each), so their product sums
// hi.hi + lo.hi + hi.lo, the Gram value to about 2^-22 relative instead of
// 2^-11 (used when 3d <= 128); xb is then the column-arrangement array
// (otherwise xb == xh). ksteps: the K steps of 16 the MMA issues.
struct TcBuffers {
    void* xh;
    void* xb;
    float* xr;
    float* cn;
    unsigned* ix;
    void* scale;
    int Kp;
    int dr;
    int split;
    int ksteps;
};
size_t tc_buffer_bytes(int64_t padded, int d);
// minmax: the per-dimension (min, max) keys of the spatial-order pass.
TcBuffers tc_prepare(void* buf, const float* xc, const float* norms, int64_t n, int d, const unsigned* perm, int nt,
                     const unsigned* minmax, cudaStream_t s);
void tc_seed(const TcBuffers& b, int t0, int mt, int d, int k, uint64_t* seed_keys, unsigned long long* kth_shared,
             cudaStream_t s);
// Workspace of the per-row lists of one sweep launch batch.
size_t tc_list_bytes(int nt, int nsplit);
// qs: the seed window (spiral positions 0..qs-1 are the seed's); plist /
// pcount (nullable): per row tile, the column tiles to visit in order (the
// small-d prune lists); without them every tile past the window is visited.
void tc_sweep(const TcBuffers& b, int nt, int t0, int mt, int nsplit, int d, int k, const unsigned* maxn,
              unsigned long long* kth_shared, uint64_t* partial, uint64_t* lists, int* status, cudaStream_t s,
              int qs = 1, const uint2* plist = nullptr, const int* pcount = nullptr);

}  // namespace culof_gb300
