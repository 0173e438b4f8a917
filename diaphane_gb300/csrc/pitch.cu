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

// Blocks walk groups of four rows (blockIdx.y is the component), threads
// along them; the four loads of a thread are issued before its stores, so a
// thread keeps four requests in flight.  No index division per element.
constexpr uint32_t kRowsPerStep = 4;

__global__ void pack_rows(const float *__restrict__ src, float *__restrict__ dst, uint32_t nx, uint32_t pitch,
                          uint64_t rows, uint64_t src_stride) {
    const float *s = src + uint64_t(blockIdx.y) * src_stride;
    float *d = dst + uint64_t(blockIdx.y) * rows * nx;
    for (uint64_t r0 = uint64_t(blockIdx.x) * kRowsPerStep; r0 < rows; r0 += uint64_t(gridDim.x) * kRowsPerStep) {
        for (uint32_t x = threadIdx.x; x < nx; x += blockDim.x) {
            float v[kRowsPerStep];
#pragma unroll
            for (uint32_t k = 0; k < kRowsPerStep; ++k)
                if (r0 + k < rows) v[k] = s[(r0 + k) * pitch + x];
#pragma unroll
            for (uint32_t k = 0; k < kRowsPerStep; ++k)
                if (r0 + k < rows) d[(r0 + k) * nx + x] = v[k];
        }
    }
}

__global__ void unpack_rows(const float *__restrict__ src, float *__restrict__ dst, uint32_t nx, uint32_t pitch,
                            uint64_t rows, uint64_t dst_stride) {
    const float *s = src + uint64_t(blockIdx.y) * rows * nx;
    float *d = dst + uint64_t(blockIdx.y) * dst_stride;
    for (uint64_t r0 = uint64_t(blockIdx.x) * kRowsPerStep; r0 < rows; r0 += uint64_t(gridDim.x) * kRowsPerStep) {
        for (uint32_t x = threadIdx.x; x < nx; x += blockDim.x) {
            float v[kRowsPerStep];
#pragma unroll
            for (uint32_t k = 0; k < kRowsPerStep; ++k)
                if (r0 + k < rows) v[k] = s[(r0 + k) * nx + x];
#pragma unroll
            for (uint32_t k = 0; k < kRowsPerStep; ++k)
                if (r0 + k < rows) d[(r0 + k) * pitch + x] = v[k];
        }
    }
}

dim3 row_grid(uint64_t rows, uint32_t components) {
    const uint64_t groups = (rows + kRowsPerStep - 1) / kRowsPerStep;
    return dim3(unsigned(groups < 16384 ? groups : 16384), components);
}

unsigned row_block(uint32_t nx) {
    const uint32_t t = (nx + 31) / 32 * 32;
    return t < 256 ? t : 256;
}

} // namespace

void launch_pack_rows(const float *src, float *dst, uint32_t nx, uint32_t pitch, uint64_t rows, uint64_t src_stride,
                      uint32_t components, cudaStream_t stream) {
    if (uint64_t(components) * rows * nx == 0) return;
    pack_rows<<<row_grid(rows, components), row_block(nx), 0, stream>>>(src, dst, nx, pitch, rows, src_stride);
}

void launch_unpack_rows(const float *src, float *dst, uint32_t nx, uint32_t pitch, uint64_t rows, uint64_t dst_stride,
                        uint32_t components, cudaStream_t stream) {
    if (uint64_t(components) * rows * nx == 0) return;
    unpack_rows<<<row_grid(rows, components), row_block(nx), 0, stream>>>(src, dst, nx, pitch, rows, dst_stride);
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
