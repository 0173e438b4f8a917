// Internal self-check of exact_div against the library's IEEE division.
// Not part of the public ABI (no header declaration); the test suite calls it
// through ctypes to show the two agree bit for bit.
#include "exact_div.cuh"

#include <cstddef>
#include <cuda_runtime.h>

namespace {

__global__ void division_check(const float *n, const float *d, float *ours, float *ieee, size_t count) {
    const size_t i = size_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= count) return;
    ours[i] = diaphane::exact_div(n[i], d[i]);
    ieee[i] = n[i] / d[i];
}

} // namespace

extern "C" int dp_internal_division_check(const float *n, const float *d, float *ours, float *ieee, size_t count) {
    float *buf = nullptr;
    if (count == 0) return 0;
    if (cudaMalloc(&buf, 4 * count * sizeof(float)) != cudaSuccess) return 1;
    int rc = 0;
    if (cudaMemcpy(buf, n, count * 4, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(buf + count, d, count * 4, cudaMemcpyHostToDevice) != cudaSuccess)
        rc = 1;
    if (!rc) {
        division_check<<<unsigned((count + 255) / 256), 256>>>(buf, buf + count, buf + 2 * count, buf + 3 * count, count);
        if (cudaDeviceSynchronize() != cudaSuccess ||
            cudaMemcpy(ours, buf + 2 * count, count * 4, cudaMemcpyDeviceToHost) != cudaSuccess ||
            cudaMemcpy(ieee, buf + 3 * count, count * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
            rc = 1;
    }
    cudaFree(buf);
    return rc;
}
