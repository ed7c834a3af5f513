/*
 * CPU oracle for exact Local Outlier Factor: TEST INFRASTRUCTURE ONLY.
 * See lof_oracle.h for the scope rule and the reference citations.
 *
 * Build flags matter: -O2 -ffp-contract=off (no silent FMA contraction and no
 * fast-math), so every float operation below rounds exactly as written.
 */
#include "lof_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

/* ---------------------------------------------------------------- helpers */

static uint32_t f2u(float f) {
    uint32_t u;
    memcpy(&u, &f, sizeof u);
    return u;
}

static float u2f(uint32_t u) {
    float f;
    memcpy(&f, &u, sizeof f);
    return f;
}

static int resolve_threads(int nthreads) {
    if (nthreads > 0) return nthreads;
    long c = sysconf(_SC_NPROCESSORS_ONLN);
    return c > 0 ? (int)c : 1;
}

/* ------------------------------------------------------------- centring */

/* preprocess.cu:31-72 computes each feature's mean (and, for normalize, the
 * population standard deviation) in double and writes (x - mean) * inv_std
 * back as float. The reduction order here is fixed: partial sums over chunks
 * of ORACLE_CENTER_CHUNK rows in ascending row order, then the partials in
 * ascending chunk order. A zero-variance feature keeps scale 1
 * (preprocess.cu:62-65). */
void oracle_center(const float* x, int64_t n, int d, int normalize, float* xc,
                   double* mean_out, double* inv_std_out) {
    const int64_t chunks = (n + ORACLE_CENTER_CHUNK - 1) / ORACLE_CENTER_CHUNK;
    for (int f = 0; f < d; ++f) {
        double total = 0.0;
        for (int64_t c = 0; c < chunks; ++c) {
            double part = 0.0;
            const int64_t end = (c + 1) * ORACLE_CENTER_CHUNK < n ? (c + 1) * ORACLE_CENTER_CHUNK : n;
            for (int64_t i = c * ORACLE_CENTER_CHUNK; i < end; ++i) part += (double)x[i * d + f];
            total += part;
        }
        const double mean = total / (double)n;
        double inv_std = 1.0;
        if (normalize) {
            double vtotal = 0.0;
            for (int64_t c = 0; c < chunks; ++c) {
                double part = 0.0;
                const int64_t end = (c + 1) * ORACLE_CENTER_CHUNK < n ? (c + 1) * ORACLE_CENTER_CHUNK : n;
                for (int64_t i = c * ORACLE_CENTER_CHUNK; i < end; ++i) {
                    const double t = (double)x[i * d + f] - mean;
                    part += t * t;
                }
                vtotal += part;
            }
            const double sd = sqrt(vtotal / (double)n);
            inv_std = (sd > 1e-12) ? 1.0 / sd : 1.0;
        }
        for (int64_t i = 0; i < n; ++i)
            xc[i * d + f] = (float)(((double)x[i * d + f] - mean) * inv_std);
        if (mean_out) mean_out[f] = mean;
        if (inv_std_out) inv_std_out[f] = inv_std;
    }
}

/* preprocess.cu:75-84: FP64 sum of squares in feature order, cast to float. */
void oracle_norms(const float* xc, int64_t n, int d, float* norms) {
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int f = 0; f < d; ++f) {
            const double v = (double)xc[i * d + f];
            s += v * v;
        }
        norms[i] = (float)s;
    }
}

/* ------------------------------------------------------------- distance */

float oracle_dist2(const float* a, const float* b, int d) {
    float s = 0.0f;
    for (int f = 0; f < d; ++f) {
        const float t = a[f] - b[f];
        s = fmaf(t, t, s);
    }
    return s;
}

/* Distances from one row to a block of columns stored feature-major
 * (colT[f * blk + j]). The per-column operation order is exactly
 * oracle_dist2's; the loop over j is what a compiler can vectorise. */
#if defined(__x86_64__) && defined(__GNUC__) && !defined(__clang__)
__attribute__((target_clones("arch=haswell", "default")))
#endif
static void dist2_block(const float* a, const float* colT, int d, int blk, float* out) {
    for (int j = 0; j < blk; ++j) out[j] = 0.0f;
    for (int f = 0; f < d; ++f) {
        const float af = a[f];
        const float* c = colT + (size_t)f * blk;
        for (int j = 0; j < blk; ++j) {
            const float t = af - c[j];
            out[j] = fmaf(t, t, out[j]);
        }
    }
}

/* ---------------------------------------------------------- k-NN select */

/* Max-heap of (d2 bits << 32 | index) keys: the k smallest seen so far. */
static void heap_sift_down(uint64_t* h, int k, int i) {
    for (;;) {
        int l = 2 * i + 1, r = l + 1, m = i;
        if (l < k && h[l] > h[m]) m = l;
        if (r < k && h[r] > h[m]) m = r;
        if (m == i) return;
        uint64_t t = h[i];
        h[i] = h[m];
        h[m] = t;
        i = m;
    }
}

static int cmp_u64(const void* a, const void* b) {
    const uint64_t x = *(const uint64_t*)a, y = *(const uint64_t*)b;
    return x < y ? -1 : (x > y);
}

/* Write one row's neighbours in the reference's slot order (knn.cu:190-224):
 * keys strictly below the k-th key's d2 by ascending index, then the ties. */
static void emit_row(uint64_t* keys, int k, int64_t n, int64_t i, int32_t* nbr_idx,
                     float* nbr_d2, float* kdist2) {
    uint32_t kth = 0;
    for (int t = 0; t < k; ++t) {
        const uint32_t b = (uint32_t)(keys[t] >> 32);
        if (b > kth) kth = b;
    }
    /* Re-key: (is_tie << 63) | (index << 32) | bits, sort, emit. */
    for (int t = 0; t < k; ++t) {
        const uint32_t b = (uint32_t)(keys[t] >> 32);
        const uint64_t j = keys[t] & 0xFFFFFFFFull;
        keys[t] = ((uint64_t)(b == kth) << 63) | (j << 32) | b;
    }
    qsort(keys, (size_t)k, sizeof(uint64_t), cmp_u64);
    for (int t = 0; t < k; ++t) {
        nbr_idx[(int64_t)t * n + i] = (int32_t)((keys[t] >> 32) & 0x7FFFFFFFull);
        nbr_d2[(int64_t)t * n + i] = u2f((uint32_t)(keys[t] & 0xFFFFFFFFull));
    }
    kdist2[i] = u2f(kth);
}

#define KNN_BLK 256

typedef struct {
    const float* xc;
    const float* colT; /* n padded to blocks of KNN_BLK, feature-major per block */
    int64_t n;
    int d, k;
    int64_t row_begin, row_end;
    int32_t* nbr_idx;
    float* nbr_d2;
    float* kdist2;
} knn_job;

/* The k smallest keys of row i against every column (unordered, in heap). */
static void select_row(const knn_job* J, int64_t i, uint64_t* heap, float* dbuf) {
    const int64_t n = J->n;
    const int d = J->d, k = J->k;
    const float* a = J->xc + i * d;
    int filled = 0;
    for (int64_t c0 = 0; c0 < n; c0 += KNN_BLK) {
        const int blk = (n - c0) < KNN_BLK ? (int)(n - c0) : KNN_BLK;
        dist2_block(a, J->colT + c0 * d, d, KNN_BLK, dbuf);
        for (int jj = 0; jj < blk; ++jj) {
            const int64_t j = c0 + jj;
            if (j == i) continue; /* a point never selects itself (knn.cu:151) */
            const uint64_t key = ((uint64_t)f2u(dbuf[jj]) << 32) | (uint64_t)j;
            if (filled < k) {
                heap[filled++] = key;
                if (filled == k)
                    for (int h = k / 2 - 1; h >= 0; --h) heap_sift_down(heap, k, h);
            } else if (key < heap[0]) {
                heap[0] = key;
                heap_sift_down(heap, k, 0);
            }
        }
    }
}

static void knn_one_row(const knn_job* J, int64_t i, uint64_t* heap, float* dbuf) {
    select_row(J, i, heap, dbuf);
    emit_row(heap, J->k, J->n, i, J->nbr_idx, J->nbr_d2, J->kdist2);
}

typedef struct {
    const knn_job* job;
    int64_t begin, end;
} knn_slice;

/* Feature-major copy of the points per block of KNN_BLK columns, zero padded. */
static float* column_blocks(const float* xc, int64_t n, int d) {
    const int64_t nblk = (n + KNN_BLK - 1) / KNN_BLK;
    float* colT = (float*)calloc((size_t)(nblk * KNN_BLK) * (size_t)d, sizeof(float));
    for (int64_t j = 0; j < n; ++j) {
        const int64_t b = j / KNN_BLK, jj = j % KNN_BLK;
        for (int f = 0; f < d; ++f) colT[b * KNN_BLK * d + (int64_t)f * KNN_BLK + jj] = xc[j * d + f];
    }
    return colT;
}

static void* knn_worker(void* p) {
    const knn_slice* s = (const knn_slice*)p;
    uint64_t* heap = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)s->job->k);
    float* dbuf = (float*)malloc(sizeof(float) * KNN_BLK);
    for (int64_t i = s->begin; i < s->end; ++i) knn_one_row(s->job, i, heap, dbuf);
    free(heap);
    free(dbuf);
    return NULL;
}

void oracle_knn_rows(const float* xc, int64_t n, int d, int k, int64_t row_begin,
                     int64_t row_end, int32_t* nbr_idx, float* nbr_d2, float* kdist2,
                     int nthreads) {
    float* colT = column_blocks(xc, n, d);
    knn_job job = {xc, colT, n, d, k, row_begin, row_end, nbr_idx, nbr_d2, kdist2};
    int nt = resolve_threads(nthreads);
    const int64_t rows = row_end - row_begin;
    if (nt > rows) nt = rows > 0 ? (int)rows : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
    knn_slice* sl = (knn_slice*)malloc(sizeof(knn_slice) * (size_t)nt);
    for (int t = 0; t < nt; ++t) {
        sl[t].job = &job;
        sl[t].begin = row_begin + rows * t / nt;
        sl[t].end = row_begin + rows * (t + 1) / nt;
        pthread_create(&th[t], NULL, knn_worker, &sl[t]);
    }
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    free(th);
    free(sl);
    free(colT);
}

/* ----------------------------------------------------------- LRD, score */

void oracle_lrd(const int32_t* nbr_idx, const float* nbr_d2, const float* kdist2,
                int64_t n, int k, float* lrd) {
    for (int64_t i = 0; i < n; ++i) {
        double sum = 0.0;
        for (int t = 0; t < k; ++t) {
            const int64_t o = (int64_t)t * n + i;
            const int32_t j = nbr_idx[o];
            sum += sqrt((double)fmaxf(kdist2[j], nbr_d2[o]));
        }
        lrd[i] = (float)(1.0 / (sum / (double)k + 1e-10));
    }
}

void oracle_score(const int32_t* nbr_idx, const float* lrd, int64_t n, int k,
                  float* scores) {
    for (int64_t i = 0; i < n; ++i) {
        const double self = (double)lrd[i];
        double sum = 0.0;
        for (int t = 0; t < k; ++t) sum += (double)lrd[nbr_idx[(int64_t)t * n + i]] / self;
        scores[i] = (float)(sum / (double)k);
    }
}

int oracle_lof(const float* x, int64_t n, int d, int k, int normalize, float* scores,
               int nthreads) {
    if (!x || n < 2 || d < 1 || k < 1 || (int64_t)k >= n) return -1;
    float* xc = (float*)malloc(sizeof(float) * (size_t)n * (size_t)d);
    int32_t* idx = (int32_t*)malloc(sizeof(int32_t) * (size_t)n * (size_t)k);
    float* d2 = (float*)malloc(sizeof(float) * (size_t)n * (size_t)k);
    float* kd = (float*)malloc(sizeof(float) * (size_t)n);
    float* lrd = (float*)malloc(sizeof(float) * (size_t)n);
    oracle_center(x, n, d, normalize, xc, NULL, NULL);
    oracle_knn_rows(xc, n, d, k, 0, n, idx, d2, kd, nthreads);
    oracle_lrd(idx, d2, kd, n, k, lrd);
    oracle_score(idx, lrd, n, k, scores);
    free(xc);
    free(idx);
    free(d2);
    free(kd);
    free(lrd);
    return 0;
}

/* ------------------------------------------------------ offset, labels */

static int cmp_f32(const void* a, const void* b) {
    const float x = *(const float*)a, y = *(const float*)b;
    return x < y ? -1 : (x > y);
}

/* numpy's 'linear' percentile on a float32 array with a Python-float q, as
 * LOF.fit calls it (__init__.py:183): q = (100 c) / 100 in double; virtual
 * index v = (n-1) q; lo = floor(v); gamma = v - lo; with a = sorted[lo],
 * b = sorted[lo+1] and diff = b - a in float32, the result is
 * b - diff * (float)(1 - gamma) when gamma >= 0.5, else a + diff * (float)gamma
 * (each product and sum rounded to float32 separately). */
double oracle_percentile_offset(const float* nof, int64_t n, double contamination) {
    float* s = (float*)malloc(sizeof(float) * (size_t)n);
    memcpy(s, nof, sizeof(float) * (size_t)n);
    qsort(s, (size_t)n, sizeof(float), cmp_f32);
    const double q = (100.0 * contamination) / 100.0;
    const double v = (double)(n - 1) * q;
    float r;
    if (v >= (double)(n - 1)) {
        r = s[n - 1];
    } else if (v < 0.0) {
        r = s[0];
    } else {
        const double lo = floor(v);
        const double gamma = v - lo;
        const float a = s[(int64_t)lo], b = s[(int64_t)lo + 1];
        const float diff = b - a;
        if (gamma >= 0.5) {
            const float w = (float)(1.0 - gamma);
            const float p = diff * w;
            r = b - p;
        } else {
            const float w = (float)gamma;
            const float p = diff * w;
            r = a + p;
        }
    }
    free(s);
    return (double)r;
}

void oracle_labels(const float* nof, int64_t n, double offset, int64_t* labels) {
    const float off = (float)offset;
    for (int64_t i = 0; i < n; ++i) labels[i] = nof[i] < off ? -1 : 1;
}

/* ------------------------------------------- reference select restatement */

void oracle_ref_select_tile(const float* tile, const float* norms, int rows,
                            int64_t row_offset, int64_t n, int k, int32_t* nbr_idx,
                            float* nbr_d2, float* kdist2) {
    uint64_t* heap = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)k);
    for (int r = 0; r < rows; ++r) {
        const int64_t self = row_offset + r;
        const float self_norm = norms[self];
        int filled = 0;
        for (int64_t j = 0; j < n; ++j) {
            const float sum = self_norm + norms[j];
            const float twice = 2.0f * tile[(int64_t)r * n + j];
            const float raw = sum - twice;
            const float d2 = (j == self || isnan(raw)) ? INFINITY : fmaxf(0.0f, raw);
            const uint64_t key = ((uint64_t)f2u(d2) << 32) | (uint64_t)j;
            if (filled < k) {
                heap[filled++] = key;
                if (filled == k)
                    for (int h = k / 2 - 1; h >= 0; --h) heap_sift_down(heap, k, h);
            } else if (key < heap[0]) {
                heap[0] = key;
                heap_sift_down(heap, k, 0);
            }
        }
        emit_row(heap, k, n, self, nbr_idx, nbr_d2, kdist2);
    }
    free(heap);
}

/* ------------------------------------------------ k-NN of a list of rows */

typedef struct {
    const knn_job* job;
    const int64_t* rows;
    int64_t m, begin, end;
} list_slice;

/* Row rows[r] goes to column r of the (k x m) outputs: emit_row with a
 * row count of m and point index r. */
static void* knn_list_worker(void* p) {
    const list_slice* s = (const list_slice*)p;
    const knn_job* J = s->job;
    uint64_t* heap = (uint64_t*)malloc(sizeof(uint64_t) * (size_t)J->k);
    float* dbuf = (float*)malloc(sizeof(float) * KNN_BLK);
    for (int64_t r = s->begin; r < s->end; ++r) {
        select_row(J, s->rows[r], heap, dbuf);
        emit_row(heap, J->k, s->m, r, J->nbr_idx, J->nbr_d2, J->kdist2);
    }
    free(heap);
    free(dbuf);
    return NULL;
}

void oracle_knn_list(const float* xc, int64_t n, int d, int k, const int64_t* rows, int64_t m,
                     int32_t* nbr_idx, float* nbr_d2, float* kdist2, int nthreads) {
    float* colT = column_blocks(xc, n, d);
    knn_job job = {xc, colT, n, d, k, 0, n, nbr_idx, nbr_d2, kdist2};
    int nt = resolve_threads(nthreads);
    if (nt > m) nt = m > 0 ? (int)m : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
    list_slice* sl = (list_slice*)malloc(sizeof(list_slice) * (size_t)nt);
    for (int t = 0; t < nt; ++t) {
        sl[t].job = &job;
        sl[t].rows = rows;
        sl[t].m = m;
        sl[t].begin = m * t / nt;
        sl[t].end = m * (t + 1) / nt;
        pthread_create(&th[t], NULL, knn_list_worker, &sl[t]);
    }
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    free(th);
    free(sl);
    free(colT);
}

/* ------------------------------------------------- FP64 brute force LOF */

/* The LOF definitions (Breunig et al. 2000) evaluated in double precision,
 * as the reference's own test oracle cpu_lof does (tests/cpp/test_culof.cu:
 * 39-80): centring in double (x - mean, divided by the population standard
 * deviation for normalize, a zero-variance feature keeping scale 1 as
 * preprocess.cu:62-65 does), Euclidean distances in double by direct
 * differences, neighbours = the k smallest (distance, index) pairs other
 * than the point itself, k-distance = distance to the k-th of them,
 * reach = max(k-distance(o), d(p, o)), lrd = 1 / (mean reach + 1e-10),
 * LOF = mean lrd(o) / lrd(p). This is the FP64 yardstick of the float32
 * engine's error, not a bit-exact restatement. */

typedef struct {
    double d2;
    int64_t j;
} pair64;

static int pair_less(pair64 a, pair64 b) { return a.d2 < b.d2 || (a.d2 == b.d2 && a.j < b.j); }

static void heap64_sift_down(pair64* h, int k, int i) {
    for (;;) {
        int l = 2 * i + 1, r = l + 1, m = i;
        if (l < k && pair_less(h[m], h[l])) m = l;
        if (r < k && pair_less(h[m], h[r])) m = r;
        if (m == i) return;
        pair64 t = h[i];
        h[i] = h[m];
        h[m] = t;
        i = m;
    }
}

static int cmp_pair64(const void* a, const void* b) {
    const pair64 x = *(const pair64*)a, y = *(const pair64*)b;
    return pair_less(x, y) ? -1 : (pair_less(y, x) ? 1 : 0);
}

static double* center_f64(const float* x, int64_t n, int d, int normalize) {
    double* xc = (double*)malloc(sizeof(double) * (size_t)n * (size_t)d);
    for (int f = 0; f < d; ++f) {
        double s = 0.0;
        for (int64_t i = 0; i < n; ++i) s += (double)x[i * d + f];
        const double mean = s / (double)n;
        double inv = 1.0;
        if (normalize) {
            double v = 0.0;
            for (int64_t i = 0; i < n; ++i) {
                const double t = (double)x[i * d + f] - mean;
                v += t * t;
            }
            const double sd = sqrt(v / (double)n);
            inv = (sd > 1e-12) ? 1.0 / sd : 1.0;
        }
        for (int64_t i = 0; i < n; ++i) xc[i * d + f] = ((double)x[i * d + f] - mean) * inv;
    }
    return xc;
}

#define F64_BLK 128

typedef struct {
    const double* xc;
    const double* colT; /* feature-major per block of F64_BLK columns */
    int64_t n;
    int d, kk;
    const int64_t* rows; /* output row r is point rows[r] (NULL: point r) */
    int64_t begin, end;  /* output rows of this worker */
    int64_t* idx;
    double* dist;
} f64_job;

static void* knn_f64_worker(void* p) {
    const f64_job* J = (const f64_job*)p;
    const int64_t n = J->n;
    const int d = J->d, kk = J->kk;
    pair64* heap = (pair64*)malloc(sizeof(pair64) * (size_t)kk);
    double dbuf[F64_BLK];
    for (int64_t r = J->begin; r < J->end; ++r) {
        const int64_t i = J->rows ? J->rows[r] : r;
        const double* a = J->xc + i * d;
        int filled = 0;
        for (int64_t c0 = 0; c0 < n; c0 += F64_BLK) {
            const int blk = (n - c0) < F64_BLK ? (int)(n - c0) : F64_BLK;
            const double* cb = J->colT + c0 * d;
            for (int jj = 0; jj < F64_BLK; ++jj) dbuf[jj] = 0.0;
            for (int f = 0; f < d; ++f) {
                const double af = a[f];
                const double* c = cb + (size_t)f * F64_BLK;
                for (int jj = 0; jj < F64_BLK; ++jj) {
                    const double t = af - c[jj];
                    dbuf[jj] += t * t;
                }
            }
            for (int jj = 0; jj < blk; ++jj) {
                const int64_t j = c0 + jj;
                if (j == i) continue;
                const pair64 e = {dbuf[jj], j};
                if (filled < kk) {
                    heap[filled++] = e;
                    if (filled == kk)
                        for (int h = kk / 2 - 1; h >= 0; --h) heap64_sift_down(heap, kk, h);
                } else if (pair_less(e, heap[0])) {
                    heap[0] = e;
                    heap64_sift_down(heap, kk, 0);
                }
            }
        }
        qsort(heap, (size_t)kk, sizeof(pair64), cmp_pair64);
        for (int t = 0; t < kk; ++t) {
            J->idx[r * kk + t] = heap[t].j;
            J->dist[r * kk + t] = sqrt(heap[t].d2);
        }
    }
    free(heap);
    return NULL;
}

static void knn_f64_rows(const double* xc, int64_t n, int d, int kk, const int64_t* row_list, int64_t m,
                         int64_t* idx, double* dist, int nthreads) {
    const int64_t nblk = (n + F64_BLK - 1) / F64_BLK;
    double* colT = (double*)calloc((size_t)(nblk * F64_BLK) * (size_t)d, sizeof(double));
    /* zero-padded columns beyond n are skipped by the blk bound */
    for (int64_t j = 0; j < n; ++j) {
        const int64_t b = j / F64_BLK, jj = j % F64_BLK;
        for (int f = 0; f < d; ++f) colT[b * F64_BLK * d + (int64_t)f * F64_BLK + jj] = xc[j * d + f];
    }
    int nt = resolve_threads(nthreads);
    if (nt > m) nt = m > 0 ? (int)m : 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nt);
    f64_job* jobs = (f64_job*)malloc(sizeof(f64_job) * (size_t)nt);
    for (int t = 0; t < nt; ++t) {
        f64_job J = {xc, colT, n, d, kk, row_list, m * t / nt, m * (t + 1) / nt, idx, dist};
        jobs[t] = J;
        pthread_create(&th[t], NULL, knn_f64_worker, &jobs[t]);
    }
    for (int t = 0; t < nt; ++t) pthread_join(th[t], NULL);
    free(th);
    free(jobs);
    free(colT);
}

void oracle_knn_f64(const float* x, int64_t n, int d, int normalize, int kk, const int64_t* rows,
                    int64_t m, int64_t* idx, double* dist, int nthreads) {
    double* xc = center_f64(x, n, d, normalize);
    knn_f64_rows(xc, n, d, kk, rows, rows ? m : n, idx, dist, nthreads);
    free(xc);
}

int oracle_lof_f64(const float* x, int64_t n, int d, int k, int normalize, double* scores, int nthreads) {
    if (!x || n < 2 || d < 1 || k < 1 || (int64_t)k >= n) return -1;
    double* xc = center_f64(x, n, d, normalize);
    int64_t* idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)n * (size_t)k);
    double* dist = (double*)malloc(sizeof(double) * (size_t)n * (size_t)k);
    double* lrd = (double*)malloc(sizeof(double) * (size_t)n);
    knn_f64_rows(xc, n, d, k, NULL, n, idx, dist, nthreads);
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int t = 0; t < k; ++t) {
            const int64_t j = idx[i * k + t];
            const double kd = dist[j * k + k - 1];
            const double dij = dist[i * k + t];
            s += kd > dij ? kd : dij;
        }
        lrd[i] = 1.0 / (s / (double)k + 1e-10);
    }
    for (int64_t i = 0; i < n; ++i) {
        double s = 0.0;
        for (int t = 0; t < k; ++t) s += lrd[idx[i * k + t]];
        scores[i] = s / ((double)k * lrd[i]);
    }
    free(xc);
    free(idx);
    free(dist);
    free(lrd);
    return 0;
}
