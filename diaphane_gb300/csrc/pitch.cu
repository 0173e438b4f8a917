// Row packing between the device layout (rows of `pitch` cells, the stride a
// TMA tensor map needs) and the reference's dense host layout (rows of nx).
//
// A strided 2-D copy between device and host moves one short row at a time;
// packing on the device first turns every read or write of a field into one
// contiguous transfer plus one pass over HBM.
#include "device.cuh"

#include <stdexcept>
#include <string>

namespace diaphane {

namespace {

__global__ void pack_rows(const float *__restrict__ src, float *__restrict__ dst, uint32_t nx, uint32_t pitch,
                          uint64_t rows, uint64_t src_stride, uint64_t total) {
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t per = rows * nx;
        const uint64_t c = i / per, r = (i % per) / nx, x = i % nx;
        dst[i] = src[c * src_stride + r * pitch + x];
    }
}

__global__ void unpack_rows(const float *__restrict__ src, float *__restrict__ dst, uint32_t nx, uint32_t pitch,
                            uint64_t rows, uint64_t dst_stride, uint64_t total) {
    for (uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x; i < total; i += uint64_t(gridDim.x) * blockDim.x) {
        const uint64_t per = rows * nx;
        const uint64_t c = i / per, r = (i % per) / nx, x = i % nx;
        dst[c * dst_stride + r * pitch + x] = src[i];
    }
}

unsigned blocks_for(uint64_t total) {
    const uint64_t b = (total + 255) / 256;
    return unsigned(b < 8192 ? (b ? b : 1) : 8192);
}

} // namespace

void launch_pack_rows(const float *src, float *dst, uint32_t nx, uint32_t pitch, uint64_t rows, uint64_t src_stride,
                      uint32_t components, cudaStream_t stream) {
    const uint64_t total = uint64_t(components) * rows * nx;
    if (total) pack_rows<<<blocks_for(total), 256, 0, stream>>>(src, dst, nx, pitch, rows, src_stride, total);
}

void launch_unpack_rows(const float *src, float *dst, uint32_t nx, uint32_t pitch, uint64_t rows, uint64_t dst_stride,
                        uint32_t components, cudaStream_t stream) {
    const uint64_t total = uint64_t(components) * rows * nx;
    if (total) unpack_rows<<<blocks_for(total), 256, 0, stream>>>(src, dst, nx, pitch, rows, dst_stride, total);
}

namespace {

void check(cudaError_t e, const char *what) {
    if (e != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
    }
}

} // namespace

void copy_fields_out(float *host, const float *device, const uint32_t n[3], uint32_t pitch, uint64_t stride,
                     int components, cudaStream_t stream) {
    const uint64_t rows = uint64_t(n[1]) * n[2], dense = rows * n[0];
    if (pitch == n[0] && stride == dense) {
        check(cudaMemcpyAsync(host, device, components * dense * sizeof(float), cudaMemcpyDeviceToHost, stream),
              "readback");
        return;
    }
    float *packed = nullptr;
    check(cudaMallocAsync(reinterpret_cast<void **>(&packed), components * dense * sizeof(float), stream), "readback");
    launch_pack_rows(device, packed, n[0], pitch, rows, stride, uint32_t(components), stream);
    check(cudaGetLastError(), "pack");
    check(cudaMemcpyAsync(host, packed, components * dense * sizeof(float), cudaMemcpyDeviceToHost, stream), "readback");
    check(cudaFreeAsync(packed, stream), "readback");
}

void copy_fields_in(float *device, const float *host, const uint32_t n[3], uint32_t pitch, uint64_t stride,
                    int components, cudaStream_t stream) {
    const uint64_t rows = uint64_t(n[1]) * n[2], dense = rows * n[0];
    if (pitch == n[0] && stride == dense) {
        check(cudaMemcpyAsync(device, host, components * dense * sizeof(float), cudaMemcpyHostToDevice, stream),
              "upload");
        return;
    }
    float *packed = nullptr;
    check(cudaMallocAsync(reinterpret_cast<void **>(&packed), components * dense * sizeof(float), stream), "upload");
    check(cudaMemcpyAsync(packed, host, components * dense * sizeof(float), cudaMemcpyHostToDevice, stream), "upload");
    launch_unpack_rows(packed, device, n[0], pitch, rows, stride, uint32_t(components), stream);
    check(cudaGetLastError(), "unpack");
    check(cudaFreeAsync(packed, stream), "upload");
}

} // namespace diaphane
