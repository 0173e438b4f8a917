// Device rasterization of a scene's shapes into the material index (u8, or
// u16 past 256 materials; Scene::material_indices, src/scene.rs:181-206):
// a cell takes the material
// of the last shape, in scene order, that contains its centre
// (Shape::contains, src/scene.rs:60-81).
//
// One block covers a segment of 128 cells of one (y, z) row.  It first
// gathers, in scene order, the shapes whose cell range (computed on the host,
// conservative by two cells) covers the segment's row and overlaps its x
// span, then every thread tests its own cell against that short list.  The
// membership tests are the host's f32 expressions compiled without
// contraction, so the index is identical to the host rasterization's.
#include "abi.hpp"
#include "device.cuh"

#include <vector>

namespace diaphane {
const Scene &scene_of(const dp_scene *s);
}

using namespace diaphane;

namespace {

constexpr int kRasterThreads = 128;
constexpr int kRasterWarps = kRasterThreads / 32;

struct RasterShape {
    dp_shape shape;
    uint32_t lo[3], hi[3]; // cells the shape can cover, per axis
};

__device__ __forceinline__ bool contains(const dp_shape &s, const float p[3]) {
    if (s.kind == DP_SHAPE_BLOCK) {
        for (int a = 0; a < 3; ++a)
            if (!(fabsf(p[a] - s.center[a]) <= 0.5f * s.size[a])) return false;
        return true;
    }
    if (s.kind == DP_SHAPE_SPHERE) {
        const float d0 = p[0] - s.center[0], d1 = p[1] - s.center[1], d2 = p[2] - s.center[2];
        float r2 = d0 * d0;
        r2 += d1 * d1;
        r2 += d2 * d2;
        return r2 <= s.radius * s.radius;
    }
    return fabsf(p[s.axis] - s.offset) <= 0.5f * s.thickness;
}

template <typename T>
__global__ void __launch_bounds__(kRasterThreads)
raster_pass(const float *__restrict__ centers, uint32_t nx, uint32_t ny, uint32_t pitch,
            const RasterShape *__restrict__ shapes, uint32_t count, T *__restrict__ out) {
    __shared__ uint32_t list[kRasterThreads];
    __shared__ uint32_t warp_hits[kRasterWarps];
    const uint32_t segments = (pitch + kRasterThreads - 1) / kRasterThreads;
    const uint32_t segment = blockIdx.x % segments;
    const uint64_t row = blockIdx.x / segments; // z * ny + y
    const uint32_t y = uint32_t(row % ny), z = uint32_t(row / ny);
    const uint32_t xa = segment * kRasterThreads, x = xa + threadIdx.x;
    const uint32_t xb = min(xa + kRasterThreads, nx) - 1; // last real cell of the segment (if xa < nx)
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    float p[3];
    p[0] = x < nx ? centers[x] : 0.0f;
    p[1] = centers[nx + y];
    p[2] = centers[nx + ny + z];
    uint32_t material = 0;
    for (uint32_t base = 0; base < count; base += kRasterThreads) {
        // The shapes of this batch that can touch the segment, kept in order.
        const uint32_t k = base + threadIdx.x;
        bool hit = false;
        if (k < count && xa < nx) {
            const RasterShape &r = shapes[k];
            hit = y >= r.lo[1] && y <= r.hi[1] && z >= r.lo[2] && z <= r.hi[2] && r.lo[0] <= xb && r.hi[0] >= xa;
        }
        const uint32_t ballot = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) warp_hits[warp] = __popc(ballot);
        __syncthreads();
        uint32_t before = 0, total = 0;
        for (int w = 0; w < kRasterWarps; ++w) {
            before += w < warp ? warp_hits[w] : 0u;
            total += warp_hits[w];
        }
        if (hit) list[before + __popc(ballot & ((1u << lane) - 1u))] = k;
        __syncthreads();
        if (x < nx)
            for (uint32_t i = 0; i < total; ++i) {
                const RasterShape &r = shapes[list[i]];
                if (x >= r.lo[0] && x <= r.hi[0] && contains(r.shape, p)) material = r.shape.material;
            }
        __syncthreads(); // the list is rewritten by the next batch
    }
    if (x < pitch) out[row * pitch + x] = x < nx ? T(material) : T(0);
}

} // namespace

namespace diaphane {

// Rasterizes into `out` (device, index_bytes per cell, rows of `pitch` >= nx
// cells, padding cells set to 0), asynchronously on `stream`.  The shape
// table and the cell centres go up through stream-ordered allocations freed
// on the same stream.
void rasterize_on_device(const Scene &s, void *out, uint32_t pitch, cudaStream_t stream) {
    const uint32_t *n = s.grid.n;
    if (pitch < n[0]) throw Error(DP_ERR_INVALID, "row pitch narrower than the grid");
    std::vector<RasterShape> table;
    for (const dp_shape &sh : s.shapes) {
        RasterShape r{};
        r.shape = sh;
        bool empty = false;
        for (int a = 0; a < 3; ++a) {
            shape_cell_range(s.grid, sh, a, r.lo[a], r.hi[a]);
            empty = empty || r.lo[a] > r.hi[a];
        }
        if (!empty) table.push_back(r);
    }
    auto check = [](cudaError_t e, const char *what) {
        if (e != cudaSuccess) {
            cudaGetLastError();
            throw Error(e == cudaErrorMemoryAllocation ? DP_ERR_OOM : DP_ERR_CUDA,
                        std::string(what) + ": " + cudaGetErrorString(e));
        }
    };
    RasterShape *d_shapes = nullptr;
    float *d_centers = nullptr;
    const size_t shape_bytes = std::max<size_t>(1, table.size()) * sizeof(RasterShape);
    check(cudaMallocAsync(reinterpret_cast<void **>(&d_shapes), shape_bytes, stream), "raster shapes");
    check(cudaMallocAsync(reinterpret_cast<void **>(&d_centers), s.centers.size() * sizeof(float), stream),
          "raster centres");
    if (!table.empty())
        check(cudaMemcpyAsync(d_shapes, table.data(), table.size() * sizeof(RasterShape), cudaMemcpyHostToDevice,
                              stream),
              "raster shapes");
    check(cudaMemcpyAsync(d_centers, s.centers.data(), s.centers.size() * sizeof(float), cudaMemcpyHostToDevice,
                          stream),
          "raster centres");
    const uint64_t segments = (pitch + kRasterThreads - 1) / kRasterThreads;
    const uint64_t blocks = segments * n[1] * n[2];
    if (blocks > 0x7fffffffull) throw Error(DP_ERR_RANGE, "grid too large for the rasterizer's launch");
    if (s.index_bytes == 1)
        raster_pass<uint8_t><<<unsigned(blocks), kRasterThreads, 0, stream>>>(
            d_centers, n[0], n[1], pitch, d_shapes, uint32_t(table.size()), static_cast<uint8_t *>(out));
    else
        raster_pass<uint16_t><<<unsigned(blocks), kRasterThreads, 0, stream>>>(
            d_centers, n[0], n[1], pitch, d_shapes, uint32_t(table.size()), static_cast<uint16_t *>(out));
    check(cudaGetLastError(), "raster launch");
    check(cudaFreeAsync(d_shapes, stream), "raster free");
    check(cudaFreeAsync(d_centers, stream), "raster free");
}

} // namespace diaphane

extern "C" dp_status dp_scene_raster(const dp_scene *scene, void *device_out, uint32_t row_pitch, void *stream) {
    return guarded([&] {
        if (!scene || !device_out) throw Error(DP_ERR_INVALID, "null argument");
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        rasterize_on_device(scene_of(scene), device_out, row_pitch ? row_pitch : scene_of(scene).grid.n[0], st);
        return DP_OK;
    });
}
