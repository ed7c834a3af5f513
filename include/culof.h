/**
 * culof_gb300 C++ API: the same declarations as the reference's public header
 * (Aminsed/cuLOF 0.2.0 include/culof.h:19-49), so C++ callers of culof::lof
 * relink against libculof_gb300.so unchanged. Implemented over the C ABI in
 * culof_c.h.
 */
#ifndef CULOF_H
#define CULOF_H

#include <stdexcept>
#include <string>
#include <vector>

#if defined(__GNUC__)
#define CULOF_CXX_API __attribute__((visibility("default")))
#else
#define CULOF_CXX_API
#endif

namespace culof {

/** Any CUDA failure (include/culof.h:22-25). */
class CULOF_CXX_API CudaError : public std::runtime_error {
public:
    explicit CudaError(const std::string& what) : std::runtime_error(what) {}
};

/** True if a usable CUDA device is present (include/culof.h:28). */
CULOF_CXX_API bool cuda_available();

/** Name, compute capability, SM count and memory of the active device (include/culof.h:31). */
CULOF_CXX_API std::string device_info();

/**
 * Local Outlier Factor scores (include/culof.h:46-47).
 *
 * @param points    host pointer to row-major (n_points x n_dims) float32 data
 * @param n_points  number of samples, >= 2
 * @param n_dims    number of features, >= 1
 * @param k         neighbours per point, 1 <= k <= n_points - 1
 * @param normalize z-score each feature before computing distances
 *
 * @throws std::invalid_argument for bad arguments, CudaError for device failure
 */
CULOF_CXX_API std::vector<float> lof(const float* points, int n_points, int n_dims, int k = 20,
                       bool normalize = false);

}  // namespace culof

#endif  // CULOF_H
