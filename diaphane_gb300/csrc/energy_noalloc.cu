// Field energy of caller-owned device arrays, with no allocation at all.
//
// For callers that cannot call cudaMalloc at the point where they need the
// energy: cudaMalloc can synchronize the whole device and can fail under
// memory pressure, so a host program that drives the solver from a loop that
// must not stall, or whose device memory is owned by another allocator, has
// no way to give dp_sim_energy its scratch on demand.  This entry point reads
// fields and tables the caller already holds, writes the two f64 sums to a
// caller-provided device buffer, and keeps its per-block partial sums in a
// fixed array compiled into the library instead of allocated memory.
//
// The array is g_energy_scratch below: 2 x 4096 f64 (64 KiB), which every GPU
// that loads the library holds until the process exits.  Each block reduces a
// fixed chunk of 65,536 cells, so a call covers at most 4096 x 65,536 = 2^28
// cells; larger grids are rejected.  Every slot a call reads is written
// earlier in the same call, so nothing has to start at zero; but all calls
// share the one array, so two calls whose kernels overlap on the GPU (other
// streams, other threads) race on it and must be serialized by the caller.
//
// The fields may have padded rows (the layout dp_sim_device_ptr hands out when
// nx is not a multiple of 4: cell (x, y, z) of component a at
// a*pitch*ny*nz + (z*ny + y)*pitch + x), and the material index may be u8 or
// u16 (scenes of more than 256 materials), with its own row pitch.  An index
// at or past the material count makes both sums NaN rather than read past the
// caller's coefficient table.
//
// Every call looks the array's device address up with cudaGetSymbolAddress
// on the current device (the symbol itself is a host stand-in, not a device
// address); the lookup allocates nothing, and doing it per call keeps the
// address right across a device reset.  The first call on a device also
// loads the library's device code there, so make it before any stream
// capture.
#include "abi.hpp"

#include <cuda_runtime.h>


namespace {

constexpr uint32_t kThreads = 256;
constexpr uint32_t kMaxBlocks = 4096;
constexpr uint64_t kCellsPerBlock = 65536;
constexpr uint64_t kMaxCells = uint64_t(kMaxBlocks) * kCellsPerBlock;

static __device__ __align__(256) double g_energy_scratch[2 * kMaxBlocks];

struct Grid3 {
    uint32_t n[3];
    uint64_t cells;          // nx*ny*nz: the cells reduced
    uint32_t field_pitch;    // row stride of the fields, in cells
    uint64_t field_stride;   // component stride: field_pitch*ny*nz
    uint32_t index_pitch;    // row stride of the material index, in cells
    uint32_t index_bytes;    // 1 (u8) or 2 (u16)
    uint32_t materials;      // entries in eps_mu
};

// energy (src/cpu.rs:654-687): every component integrated over its own box,
// ½·εr·E² over primary(a)·dual(b)·dual(c) and ½·μr·H² over
// dual(a)·primary(b)·primary(c), accumulated in f64.
__global__ void __launch_bounds__(kThreads) energy_partials(const float *__restrict__ e, const float *__restrict__ h,
                                                            const void *__restrict__ material,
                                                            const float *__restrict__ eps_mu,
                                                            const float *__restrict__ primary,
                                                            const float *__restrict__ dual, Grid3 g,
                                                            double *scratch) {
    const uint32_t offset[3] = {0, g.n[0], g.n[0] + g.n[1]};
    const uint64_t begin = uint64_t(blockIdx.x) * kCellsPerBlock;
    const uint64_t end = begin + kCellsPerBlock < g.cells ? begin + kCellsPerBlock : g.cells;
    const uint8_t *index8 = static_cast<const uint8_t *>(material);
    const uint16_t *index16 = static_cast<const uint16_t *>(material);
    double ee = 0.0, em = 0.0;
    bool bad = false;
    for (uint64_t i = begin + threadIdx.x; i < end; i += kThreads) {
        uint32_t c[3];
        c[0] = uint32_t(i % g.n[0]);
        const uint64_t row = i / g.n[0]; // z*ny + y
        c[1] = uint32_t(row % g.n[1]);
        c[2] = uint32_t(row / g.n[1]);
        const uint64_t at = row * g.field_pitch + c[0];
        const uint64_t mi = row * g.index_pitch + c[0];
        const uint32_t m = g.index_bytes == 2 ? uint32_t(index16[mi]) : uint32_t(index8[mi]);
        if (m >= g.materials) {
            bad = true;
            continue;
        }
        const float er = eps_mu[2 * m], mr = eps_mu[2 * m + 1];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int b = (a + 1) % 3, cc = (a + 2) % 3;
            const float ev = e[uint64_t(a) * g.field_stride + at];
            const float hv = h[uint64_t(a) * g.field_stride + at];
            const double volume_e = double(primary[offset[a] + c[a]]) * double(dual[offset[b] + c[b]]) *
                                    double(dual[offset[cc] + c[cc]]);
            const double volume_h = double(dual[offset[a] + c[a]]) * double(primary[offset[b] + c[b]]) *
                                    double(primary[offset[cc] + c[cc]]);
            ee += 0.5 * volume_e * double(er * ev * ev);
            em += 0.5 * volume_h * double(mr * hv * hv);
        }
    }
    if (bad) ee = em = __longlong_as_double(0x7ff8000000000000ll); // NaN: an index past the table
    __shared__ double se[kThreads], sm[kThreads];
    se[threadIdx.x] = ee;
    sm[threadIdx.x] = em;
    __syncthreads();
    for (uint32_t w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            se[threadIdx.x] += se[threadIdx.x + w];
            sm[threadIdx.x] += sm[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        scratch[2 * blockIdx.x] = se[0];
        scratch[2 * blockIdx.x + 1] = sm[0];
    }
}

// Sums the partials of `blocks` blocks in a fixed order into out[0], out[1].
__global__ void __launch_bounds__(kThreads) energy_finish(const double *scratch, uint32_t blocks, double *out) {
    double ee = 0.0, em = 0.0;
    for (uint32_t b = threadIdx.x; b < blocks; b += kThreads) {
        ee += scratch[2 * b];
        em += scratch[2 * b + 1];
    }
    __shared__ double se[kThreads], sm[kThreads];
    se[threadIdx.x] = ee;
    sm[threadIdx.x] = em;
    __syncthreads();
    for (uint32_t w = kThreads / 2; w > 0; w >>= 1) {
        if (threadIdx.x < w) {
            se[threadIdx.x] += se[threadIdx.x + w];
            sm[threadIdx.x] += sm[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        out[0] = se[0];
        out[1] = sm[0];
    }
}

void check(cudaError_t err, const char *what) {
    if (err != cudaSuccess) {
        cudaGetLastError();
        throw diaphane::Error(DP_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(err));
    }
}

// The device address of g_energy_scratch on the current device.
double *scratch_address() {
    void *p = nullptr;
    check(cudaGetSymbolAddress(&p, g_energy_scratch), "cudaGetSymbolAddress");
    return static_cast<double *>(p);
}

} // namespace

extern "C" dp_status dp_energy_noalloc(const float *electric, const float *magnetic, uint32_t field_pitch,
                                       const void *material_index, uint32_t index_bytes, uint32_t index_pitch,
                                       const float *eps_mu, uint32_t material_count, const float *primary,
                                       const float *dual, const uint32_t extent[3], double *out, void *stream) {
    return diaphane::guarded([&] {
        if (!electric || !magnetic || !material_index || !eps_mu || !primary || !dual || !extent || !out)
            throw diaphane::Error(DP_ERR_INVALID, "null argument");
        Grid3 g{};
        for (int a = 0; a < 3; ++a) g.n[a] = extent[a];
        g.cells = uint64_t(extent[0]) * extent[1] * extent[2];
        if (g.cells == 0) throw diaphane::Error(DP_ERR_INVALID, "empty grid");
        if (g.cells > kMaxCells)
            throw diaphane::Error(DP_ERR_RANGE, "dp_energy_noalloc covers at most 2^28 cells (its fixed scratch holds "
                                                "4096 partial sums of 65536 cells each); use dp_sim_energy");
        g.field_pitch = field_pitch ? field_pitch : extent[0];
        g.index_pitch = index_pitch ? index_pitch : extent[0];
        if (g.field_pitch < extent[0] || g.index_pitch < extent[0])
            throw diaphane::Error(DP_ERR_INVALID, "a row pitch is narrower than the grid");
        if (index_bytes != 1 && index_bytes != 2)
            throw diaphane::Error(DP_ERR_INVALID, "index_bytes must be 1 (u8) or 2 (u16)");
        if (material_count == 0) throw diaphane::Error(DP_ERR_INVALID, "no materials");
        g.index_bytes = index_bytes;
        g.materials = material_count;
        g.field_stride = uint64_t(g.field_pitch) * extent[1] * extent[2];
        double *scratch = scratch_address();
        const uint32_t blocks = uint32_t((g.cells + kCellsPerBlock - 1) / kCellsPerBlock);
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        energy_partials<<<blocks, kThreads, 0, st>>>(electric, magnetic, material_index, eps_mu, primary, dual, g,
                                                     scratch);
        energy_finish<<<1, kThreads, 0, st>>>(scratch, blocks, out);
        check(cudaGetLastError(), "energy launch");
        return DP_OK;
    });
}
