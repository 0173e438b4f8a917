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
// The array is g_energy_scratch below: 2 × 4096 f64 (64 KiB), which every GPU
// that loads the library holds until the process exits.  Each block reduces a
// fixed chunk of 65,536 cells, so a call covers at most 4096 × 65,536 = 2^28
// cells; larger grids are rejected.  Every slot a call reads is written
// earlier in the same call, so nothing has to start at zero; but all calls
// share the one array, so two calls whose kernels overlap on the GPU (other
// streams, other threads) race on it and must be serialized by the caller.
// The first call on a device looks the array's device address up with
// cudaGetSymbolAddress (the symbol itself is a host stand-in, not a device
// address); that first call should come before any stream capture.
#include "abi.hpp"

#include <cuda_runtime.h>

#include <mutex>

namespace {

constexpr uint32_t kThreads = 256;
constexpr uint32_t kMaxBlocks = 4096;
constexpr uint64_t kCellsPerBlock = 65536;
constexpr uint64_t kMaxCells = uint64_t(kMaxBlocks) * kCellsPerBlock;
constexpr int kMaxDevices = 64;

static __device__ __align__(256) double g_energy_scratch[2 * kMaxBlocks];

// Host-side addresses of g_energy_scratch, one per device, filled on the first
// call made with that device current.  The symbol itself is only a host
// stand-in and must never be handed to a kernel.
std::mutex g_setup_mutex;
double *g_scratch_address[kMaxDevices] = {};

struct Grid3 {
    uint32_t n[3];
    uint64_t cells;
};

// energy (src/cpu.rs:654-687): every component integrated over its own box,
// ½·εr·E² over primary(a)·dual(b)·dual(c) and ½·μr·H² over
// dual(a)·primary(b)·primary(c), accumulated in f64.
__global__ void __launch_bounds__(kThreads) energy_partials(const float *__restrict__ e, const float *__restrict__ h,
                                                            const uint8_t *__restrict__ material,
                                                            const float *__restrict__ eps_mu,
                                                            const float *__restrict__ primary,
                                                            const float *__restrict__ dual, Grid3 g,
                                                            double *scratch) {
    const uint32_t offset[3] = {0, g.n[0], g.n[0] + g.n[1]};
    const uint64_t begin = uint64_t(blockIdx.x) * kCellsPerBlock;
    const uint64_t end = begin + kCellsPerBlock < g.cells ? begin + kCellsPerBlock : g.cells;
    double ee = 0.0, em = 0.0;
    for (uint64_t i = begin + threadIdx.x; i < end; i += kThreads) {
        uint32_t c[3];
        c[0] = uint32_t(i % g.n[0]);
        const uint64_t t = i / g.n[0];
        c[1] = uint32_t(t % g.n[1]);
        c[2] = uint32_t(t / g.n[1]);
        const uint32_t m = material[i];
        const float er = eps_mu[2 * m], mr = eps_mu[2 * m + 1];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const int b = (a + 1) % 3, cc = (a + 2) % 3;
            const float ev = e[uint64_t(a) * g.cells + i];
            const float hv = h[uint64_t(a) * g.cells + i];
            const double volume_e = double(primary[offset[a] + c[a]]) * double(dual[offset[b] + c[b]]) *
                                    double(dual[offset[cc] + c[cc]]);
            const double volume_h = double(dual[offset[a] + c[a]]) * double(primary[offset[b] + c[b]]) *
                                    double(primary[offset[cc] + c[cc]]);
            ee += 0.5 * volume_e * double(er * ev * ev);
            em += 0.5 * volume_h * double(mr * hv * hv);
        }
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

// The device address of g_energy_scratch on the current device, looked up
// once per device.
double *scratch_address() {
    int device = -1;
    check(cudaGetDevice(&device), "cudaGetDevice");
    if (device < 0 || device >= kMaxDevices) throw diaphane::Error(DP_ERR_UNSUPPORTED, "device ordinal out of range");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_address[device]) {
        void *p = nullptr;
        check(cudaGetSymbolAddress(&p, g_energy_scratch), "cudaGetSymbolAddress");
        g_scratch_address[device] = static_cast<double *>(p);
    }
    return g_scratch_address[device];
}

} // namespace

extern "C" dp_status dp_energy_noalloc(const float *electric, const float *magnetic, const uint8_t *material_index,
                                       const float *eps_mu, const float *primary, const float *dual,
                                       const uint32_t extent[3], double *out, void *stream) {
    return diaphane::guarded([&] {
        if (!electric || !magnetic || !material_index || !eps_mu || !primary || !dual || !extent || !out)
            throw diaphane::Error(DP_ERR_INVALID, "null argument");
        Grid3 g{{extent[0], extent[1], extent[2]}, uint64_t(extent[0]) * extent[1] * extent[2]};
        if (g.cells == 0) throw diaphane::Error(DP_ERR_INVALID, "empty grid");
        if (g.cells > kMaxCells)
            throw diaphane::Error(DP_ERR_RANGE, "dp_energy_noalloc covers at most 2^28 cells (its fixed scratch holds "
                                                "4096 partial sums of 65536 cells each); use dp_sim_energy");
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
