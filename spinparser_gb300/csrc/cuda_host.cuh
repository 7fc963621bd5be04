// Host-side CUDA helpers of the XYZ and TRI cores: status check, device allocation, host to
// device copy and the grid of elementwise kernels.
#pragma once

#include <cuda_runtime.h>
#include <algorithm>
#include <string>
#include "host/capi_common.hpp"

namespace spn {
namespace cuh {

inline void check_cuda(cudaError_t e, const char *what) {
    if (e != cudaSuccess) throw Error(ErrorType::Cuda, std::string(what) + ": " + cudaGetErrorString(e));
}

// count elements of T (at least one) plus 16 bytes of slack for vector tail reads
template <class T>
T *dalloc(size_t count, const char *what) {
    void *p = nullptr;
    check_cuda(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T) + 16), what);
    return static_cast<T *>(p);
}

template <class T>
void h2d(T *dst, const T *src, size_t count, cudaStream_t s) {
    if (count) check_cuda(cudaMemcpyAsync(dst, src, count * sizeof(T), cudaMemcpyHostToDevice, s), "cudaMemcpyAsync H2D");
}

// blocks of 256 threads for an elementwise kernel over n items (grid-stride beyond 4096 blocks)
inline int copy_grid(long long n) { return int(std::min<long long>((n + 255) / 256, 4096)); }

// The frequency mesh of a diagnostic read: 2 <= n <= max_n positive, strictly ascending values.
inline void check_mesh(const float *pos, int n, int max_n) {
    if (!pos || n < 2 || n > max_n)
        throw Error(ErrorType::Argument, "mesh: need 2 <= n <= " + std::to_string(max_n) + " values");
    for (int i = 0; i < n; ++i)
        if (!(pos[i] > 0.0f) || (i > 0 && !(pos[i] > pos[i - 1])))
            throw Error(ErrorType::Argument, "mesh: values must be positive and strictly ascending");
}

// The index of the mesh value |w| (the channel's own frequency of an access buffer).
inline int mesh_index_of(const float *pos, int n, float w) {
    const float a = w < 0.0f ? -w : w;
    for (int i = 0; i < n; ++i)
        if (pos[i] == a) return i;
    throw Error(ErrorType::Argument, "the channel's own frequency must be a mesh value");
}

}  // namespace cuh
}  // namespace spn
