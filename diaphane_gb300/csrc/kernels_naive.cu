// One-thread-per-cell kernels: the H pass, the E pass, an injection pass,
// the intensity pass, and the energy / finiteness reductions; the H, E,
// injection and energy passes also in double for the FP64 instance.
//
// These mirror the reference step's structure (src/cpu.rs:174-198) pass for
// pass and are kept for four jobs: the exact inverse step (reverse_by), the
// fallback for scenes the fused kernel does not cover, an independent second
// implementation the fused kernel is checked against, and the FP64 instance.
#include "device.cuh"
#include "exact_div.cuh"

#include <stdexcept>

namespace diaphane {

namespace {

constexpr int kThreads = 256;

// The cell of the H and E passes: block (row, x-chunk), thread along x; one
// 32-bit division per thread.  False past nx.
__device__ __forceinline__ bool cell_of(const DeviceScene &s, uint32_t c[3], uint64_t &i) {
    c[0] = blockIdx.y * kThreads + threadIdx.x;
    const uint32_t row = blockIdx.x;
    c[1] = row % s.n[1];
    c[2] = row / s.n[1];
    i = uint64_t(row) * s.pitch + c[0];
    return c[0] < s.n[0];
}

// ((1 -/+ loss) v -/+ g curl) / (1 +/- loss), the reference's semi-implicit
// update: a lossless cell's is v -/+ g curl exactly (1 -/+ 0 = 1, x / 1 = x),
// and an f32 lossy one divides without the library's slow path for tiny
// numerators (exact_div).
template <typename T> __device__ __forceinline__ T semi_implicit(T old, T loss, T drive) {
    if (loss == T(0)) return old + drive;
    const T n = (T(1) - loss) * old + drive;
    if constexpr (sizeof(T) == 4) return exact_div(n, T(1) + loss);
    else return n / (T(1) + loss);
}
// The inverse update (reversal runs only on lossless scenes, so the division
// is not reached there; 1 - loss can be below 1, outside exact_div's range).
template <typename T> __device__ __forceinline__ T semi_implicit_back(T old, T loss, T drive) {
    if (loss == T(0)) return old + drive;
    return ((T(1) + loss) * old + drive) / (T(1) - loss);
}

// Absorber sample: section 0 holds integer positions, section 1 half ones.
__device__ __forceinline__ float profile(const float *absorber, uint32_t span, const uint32_t offset[3], int axis,
                                         uint32_t coord, bool half) {
    return __ldg(&absorber[(half ? span : 0) + offset[axis] + coord]);
}

// update_magnetic (src/cpu.rs:283-376) and reverse_magnetic (:490-572) for
// every cell at once: the bulk sweep and the two high-wall planes are the same
// expression with the missing forward neighbour read as the wall's zero.  In
// double (T) the gains, losses and coefficients are the f32 setup values
// promoted, and the loss is summed in f32 as the setup tables are.
template <typename T, bool Reverse>
__global__ void __launch_bounds__(kThreads) magnetic_pass(DeviceScene s, const T *__restrict__ e,
                                                          T *__restrict__ h) {
    uint32_t c[3];
    uint64_t i;
    if (!cell_of(s, c, i)) return;
    const uint64_t stride[3] = {1, s.pitch, uint64_t(s.pitch) * s.n[1]};
    const uint32_t offset[3] = {0, s.n[0], s.n[0] + s.n[1]};
    const uint32_t span = s.n[0] + s.n[1] + s.n[2];
    const float4 k = s.coeff[material_of(s, i)];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int b = (a + 1) % 3, cc = (a + 2) % 3;
        const T *ec = e + uint64_t(cc) * s.cells;
        const T *eb = e + uint64_t(b) * s.cells;
        const T next_c = c[b] + 1 < s.n[b] ? ec[i + stride[b]] : T(0);
        const T next_b = c[cc] + 1 < s.n[cc] ? eb[i + stride[cc]] : T(0);
        const T curl = T(__ldg(&s.mgain[offset[b] + c[b]])) * (next_c - ec[i]) -
                       T(__ldg(&s.mgain[offset[cc] + c[cc]])) * (next_b - eb[i]);
        // magnetic_row: the integer profile along a, half along the others.
        const float row = profile(s.absorber, span, offset, 1, c[1], a != 1) +
                          profile(s.absorber, span, offset, 2, c[2], a != 2);
        const T loss = T((k.w + row) + profile(s.absorber, span, offset, 0, c[0], a != 0));
        T *target = h + uint64_t(a) * s.cells + i;
        const T old = *target;
        if (Reverse) *target = semi_implicit_back(old, loss, T(k.z) * curl);
        else *target = semi_implicit(old, loss, -(T(k.z) * curl));
    }
}

// update_electric (src/cpu.rs:380-434) and reverse_electric (:441-487).
// Index 0 along b or c is never written: the low-wall conductor.
template <typename T, bool Reverse>
__global__ void __launch_bounds__(kThreads) electric_pass(DeviceScene s, const T *__restrict__ h,
                                                          T *__restrict__ e) {
    uint32_t c[3];
    uint64_t i;
    if (!cell_of(s, c, i)) return;
    const uint64_t stride[3] = {1, s.pitch, uint64_t(s.pitch) * s.n[1]};
    const uint32_t offset[3] = {0, s.n[0], s.n[0] + s.n[1]};
    const uint32_t span = s.n[0] + s.n[1] + s.n[2];
    const float4 k = s.coeff[material_of(s, i)];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int b = (a + 1) % 3, cc = (a + 2) % 3;
        if (c[b] == 0 || c[cc] == 0) continue;
        const T *hc = h + uint64_t(cc) * s.cells;
        const T *hb = h + uint64_t(b) * s.cells;
        const T curl = T(__ldg(&s.egain[offset[b] + c[b]])) * (hc[i] - hc[i - stride[b]]) -
                       T(__ldg(&s.egain[offset[cc] + c[cc]])) * (hb[i] - hb[i - stride[cc]]);
        // electric_row: the half profile along a, integer along the others.
        const float row = profile(s.absorber, span, offset, 1, c[1], a == 1) +
                          profile(s.absorber, span, offset, 2, c[2], a == 2);
        const T loss = T((k.y + row) + profile(s.absorber, span, offset, 0, c[0], a == 0));
        T *target = e + uint64_t(a) * s.cells + i;
        const T old = *target;
        if (Reverse) *target = semi_implicit_back(old, loss, -(T(k.x) * curl));
        else *target = semi_implicit(old, loss, T(k.x) * curl);
    }
}

// One soft injection over its box (fdtd.wgsl inject, src/cpu.rs:618-629);
// `value` is the drive with its sign applied.
template <typename T>
__global__ void __launch_bounds__(kThreads) inject_pass(DeviceScene s, Fields<T> f, DeviceInjection inj, T value,
                                                        const T *__restrict__ profiles) {
    const uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
    const uint64_t count = uint64_t(inj.extent[0]) * inj.extent[1] * inj.extent[2];
    if (i >= count) return;
    const uint32_t dx = uint32_t(i % inj.extent[0]);
    const uint64_t t = i / inj.extent[0];
    const uint32_t dy = uint32_t(t % inj.extent[1]);
    const uint32_t dz = uint32_t(t / inj.extent[1]);
    const uint64_t cell = (uint64_t(inj.origin[2] + dz) * s.n[1] + (inj.origin[1] + dy)) * s.pitch + inj.origin[0] + dx;
    const T weight = injection_weight<T>(inj, s.weights, profiles, inj.origin[0] + dx, inj.origin[1] + dy,
                                         inj.origin[2] + dz, i);
    T *field = (inj.magnetic ? f.h : f.e) + uint64_t(inj.component) * s.cells;
    field[cell] += value * weight;
}

// I += Ex² + Ey² + Ez² (src/cpu.rs:186-196).
__global__ void __launch_bounds__(kThreads) intensity_pass(DeviceScene s, const float *__restrict__ e,
                                                           float *__restrict__ intensity) {
    const uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
    if (i >= s.cells) return;
    const float ex = e[i], ey = e[s.cells + i], ez = e[2 * s.cells + i];
    float sum = ex * ex;
    sum += ey * ey;
    sum += ez * ez;
    intensity[i] += sum;
}

// energy (src/cpu.rs:654-687): each component integrated over its own box,
// accumulated in f64.  One partial pair per block; the host adds them.
template <typename T>
__global__ void __launch_bounds__(kThreads) energy_pass(DeviceScene s, Fields<T> f, const float *__restrict__ primary,
                                                        const float *__restrict__ dual,
                                                        const float2 *__restrict__ eps_mu, double *partials) {
    // A component's volume is a product of one width per axis, so it splits
    // into an x factor and a row (y, z) factor: E_x takes primary x, dual y
    // and z; E_y and E_z dual x; H the other way round.  One warp per row sums
    // x factor × energy in double along the row, and the row factors multiply
    // once per row: a handful of double operations per cell instead of the
    // three-way volume products (the device's f64 rate is what bounds this).
    constexpr int kWarps = kThreads / 32;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t nx = s.n[0], ny = s.n[1], oy = s.n[0], oz = s.n[0] + s.n[1];
    const uint64_t rows = uint64_t(ny) * s.n[2];
    double ee = 0.0, em = 0.0;
    for (uint64_t row = uint64_t(blockIdx.x) * kWarps + warp; row < rows; row += uint64_t(gridDim.x) * kWarps) {
        double sum[6] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
        for (uint32_t x = lane; x < nx; x += 32) {
            const uint64_t i = row * s.pitch + x;
            const float2 m = eps_mu[material_of(s, i)];
            const double px = double(__ldg(&primary[x])), dx = double(__ldg(&dual[x]));
            double qe[3], qh[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const T ev = f.e[uint64_t(a) * s.cells + i], hv = f.h[uint64_t(a) * s.cells + i];
                qe[a] = double(T(m.x) * ev * ev);
                qh[a] = double(T(m.y) * hv * hv);
            }
            // Fused multiply-adds in double (the build contracts nothing by
            // itself): one rounding per term, well inside the 1e-9 the
            // energy is checked to.
            sum[0] = fma(px, qe[0], sum[0]);
            sum[1] = fma(dx, qe[1], sum[1]);
            sum[2] = fma(dx, qe[2], sum[2]);
            sum[3] = fma(dx, qh[0], sum[3]);
            sum[4] = fma(px, qh[1], sum[4]);
            sum[5] = fma(px, qh[2], sum[5]);
        }
        const uint32_t y = uint32_t(row % ny), z = uint32_t(row / ny);
        const double py = double(primary[oy + y]), dy = double(dual[oy + y]);
        const double pz = double(primary[oz + z]), dz = double(dual[oz + z]);
        ee += 0.5 * ((dy * dz) * sum[0] + (py * dz) * sum[1] + (pz * dy) * sum[2]);
        em += 0.5 * ((py * pz) * sum[3] + (dy * pz) * sum[4] + (dz * py) * sum[5]);
    }
    __shared__ double se[kThreads], sm[kThreads];
    se[threadIdx.x] = ee;
    sm[threadIdx.x] = em;
    __syncthreads();
    for (int w = kThreads / 2; w > 0; w >>= 1) {
        if (int(threadIdx.x) < w) {
            se[threadIdx.x] += se[threadIdx.x + w];
            sm[threadIdx.x] += sm[threadIdx.x + w];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        partials[2 * blockIdx.x] = se[0];
        partials[2 * blockIdx.x + 1] = sm[0];
    }
}

// energy_density (src/cpu.rs:689-703): ½(E² + H²) summed over the three
// components, per cell, into dense rows.
__global__ void __launch_bounds__(kThreads) energy_density_pass(DeviceScene s, FieldSet f, float *__restrict__ out) {
    const uint64_t dense = uint64_t(s.n[0]) * s.n[1] * s.n[2];
    const uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x;
    if (i >= dense) return;
    const uint64_t at = (i / s.n[0]) * s.pitch + i % s.n[0];
    float density = 0.0f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float e = f.e[uint64_t(a) * s.cells + at], h = f.h[uint64_t(a) * s.cells + at];
        density += 0.5f * (e * e + h * h);
    }
    out[i] = density;
}

// is_finite (src/cpu.rs:707-713): any non-finite value clears the flag.
// 16-byte loads (the field sets are 16-byte aligned), the few values past the
// last whole quad checked one by one.
__global__ void __launch_bounds__(kThreads) finite_pass(DeviceScene s, FieldSet f, int32_t *flag) {
    const uint64_t total = 3 * s.cells, quads = total / 4;
    const float4 *e = reinterpret_cast<const float4 *>(f.e), *h = reinterpret_cast<const float4 *>(f.h);
    bool ok = true;
    for (uint64_t i = uint64_t(blockIdx.x) * kThreads + threadIdx.x; i < quads; i += uint64_t(gridDim.x) * kThreads) {
        const float4 a = __ldg(e + i), b = __ldg(h + i);
        ok = ok && isfinite(a.x) && isfinite(a.y) && isfinite(a.z) && isfinite(a.w) && isfinite(b.x) &&
             isfinite(b.y) && isfinite(b.z) && isfinite(b.w);
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        for (uint64_t i = 4 * quads; i < total; ++i) ok = ok && isfinite(f.e[i]) && isfinite(f.h[i]);
    if (!__all_sync(0xffffffffu, ok) && (threadIdx.x & 31) == 0) atomicExch(flag, 0);
}

uint32_t blocks_for(uint64_t n) { return uint32_t((n + kThreads - 1) / kThreads); }

} // namespace

namespace {

// Blocks: one per (row, 256-cell chunk of the row).
dim3 pass_grid(const DeviceScene &s) {
    const uint64_t rows = uint64_t(s.n[1]) * s.n[2];
    if (rows > 0x7fffffffull) throw std::runtime_error("grid has too many rows for the per-cell passes");
    return dim3(unsigned(rows), (s.n[0] + kThreads - 1) / kThreads);
}

template <typename T> void magnetic(const DeviceScene &s, Fields<T> f, bool reverse, cudaStream_t stream) {
    if (reverse)
        magnetic_pass<T, true><<<pass_grid(s), kThreads, 0, stream>>>(s, f.e, f.h);
    else
        magnetic_pass<T, false><<<pass_grid(s), kThreads, 0, stream>>>(s, f.e, f.h);
}

template <typename T> void electric(const DeviceScene &s, Fields<T> f, bool reverse, cudaStream_t stream) {
    if (reverse)
        electric_pass<T, true><<<pass_grid(s), kThreads, 0, stream>>>(s, f.h, f.e);
    else
        electric_pass<T, false><<<pass_grid(s), kThreads, 0, stream>>>(s, f.h, f.e);
}

template <typename T> void inject(const DeviceScene &s, Fields<T> f, const DeviceInjection &inj, T value,
                                  const T *profiles, cudaStream_t stream) {
    const uint64_t count = uint64_t(inj.extent[0]) * inj.extent[1] * inj.extent[2];
    if (count == 0) return;
    inject_pass<T><<<blocks_for(count), kThreads, 0, stream>>>(s, f, inj, value, profiles);
}

} // namespace

void launch_naive_magnetic(const DeviceScene &s, FieldSet f, bool reverse, cudaStream_t stream) {
    magnetic(s, f, reverse, stream);
}
void launch_naive_magnetic(const DeviceScene &s, FieldSet64 f, bool reverse, cudaStream_t stream) {
    magnetic(s, f, reverse, stream);
}
void launch_naive_electric(const DeviceScene &s, FieldSet f, bool reverse, cudaStream_t stream) {
    electric(s, f, reverse, stream);
}
void launch_naive_electric(const DeviceScene &s, FieldSet64 f, bool reverse, cudaStream_t stream) {
    electric(s, f, reverse, stream);
}

// sign · value is exact (sign is ±1), so the f32 drive is the reference's.
void launch_inject(const DeviceScene &s, FieldSet f, const DeviceInjection &inj, float sign, const float *profiles,
                   cudaStream_t stream) {
    inject(s, f, inj, sign * inj.value, profiles, stream);
}
void launch_inject(const DeviceScene &s, FieldSet64 f, const DeviceInjection &inj, double value,
                   const double *profiles, cudaStream_t stream) {
    inject(s, f, inj, value, profiles, stream);
}

void launch_intensity(const DeviceScene &s, const float *e, float *intensity, cudaStream_t stream) {
    intensity_pass<<<blocks_for(s.cells), kThreads, 0, stream>>>(s, e, intensity);
}

uint32_t energy_blocks(uint64_t cells) {
    uint64_t b = blocks_for(cells);
    return uint32_t(b < 1024 ? b : 1024);
}

void launch_energy(const DeviceScene &s, FieldSet f, const float *primary, const float *dual, const float2 *eps_mu,
                   double *partials, uint32_t blocks, cudaStream_t stream) {
    energy_pass<float><<<blocks, kThreads, 0, stream>>>(s, f, primary, dual, eps_mu, partials);
}
void launch_energy(const DeviceScene &s, FieldSet64 f, const float *primary, const float *dual, const float2 *eps_mu,
                   double *partials, uint32_t blocks, cudaStream_t stream) {
    energy_pass<double><<<blocks, kThreads, 0, stream>>>(s, f, primary, dual, eps_mu, partials);
}

void launch_energy_density(const DeviceScene &s, FieldSet f, float *dense_out, cudaStream_t stream) {
    energy_density_pass<<<blocks_for(uint64_t(s.n[0]) * s.n[1] * s.n[2]), kThreads, 0, stream>>>(s, f, dense_out);
}

void launch_finite(const DeviceScene &s, FieldSet f, int32_t *flag, cudaStream_t stream) {
    uint64_t b = blocks_for(3 * s.cells / 4 + 1);
    finite_pass<<<uint32_t(b < 4864 ? b : 4864), kThreads, 0, stream>>>(s, f, flag);
}

} // namespace diaphane
