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

}  // namespace cuh
}  // namespace spn
