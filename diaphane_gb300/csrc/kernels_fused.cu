// The fused Yee step: H and E of a whole time step in one pass over HBM.
//
// Why one pass works.  The H update at plane z reads E at planes z and z+1
// (forward differences); the E update at plane z reads the *new* H at planes
// z and z-1 (backward differences).  Walking z upward, a CTA can therefore
// finish H(z), then E(z), holding new H(z-1) in registers.  Two things make
// that legal without grid-wide synchronisation:
//   * ping-pong field sets: every read comes from the `in` set and every
//     write goes to the `out` set, so no CTA can overwrite a value another
//     CTA still needs (the reference updates in place because its two passes
//     are separated by a barrier; a fused pass cannot be);
//   * halo recompute: E at the tile's low x column and low y row needs new H
//     one cell outside the tile, so a ninth warp recomputes H there from the
//     same inputs instead of waiting for the neighbouring CTA.
// Each cell's six components are then read once and written once per step:
// the 48 B/cell of the reference's own accounting (src/gpu.rs:381-388).
//
// Data movement.  z-planes of the tile stream through a 3-slot ring in
// shared memory filled by TMA (cp.async.bulk.tensor): E with one cell of
// halo on every side (out-of-range cells arrive as zero, which is exactly the
// perfect conductor's tangential E beyond the high walls), H with the low
// halo, and the u8 material index.  The coefficient table sits in shared
// memory.  Gains and absorber profiles along x stay in registers; along y and
// z they are per-row and per-plane scalars.
//
// Arithmetic.  Each component is the reference's expression in the
// reference's order (src/cpu.rs:323-330, 422-429), compiled without FMA
// contraction; a cell whose total loss is exactly zero takes the shortcut
// `h - g*curl`, which is the same IEEE result as `((1-0)h - g*curl)/(1+0)`.
// Sources are applied to each freshly computed value in the reference's
// order (src/cpu.rs:606-633), halo cells included, and intensity is summed
// from the final E (src/cpu.rs:186-196).  The result is bit-identical to the
// reference's two-pass f32 step.
#include "device.cuh"

#include <cuda.h>

#include <cstdio>
#include <stdexcept>
#include <string>

namespace diaphane {

namespace {

constexpr int kTileY = 8;                 // rows per tile, one compute warp each
constexpr int kWarps = kTileY + 1;        // + the halo warp
constexpr int kThreads = kWarps * 32;
constexpr int kSlots = 3;                 // plane ring depth
constexpr int kMaxMaterials = 256;
constexpr long long kWaitCycles = 1ll << 32; // ~2 s at 2 GHz, then give up

template <int CX> struct Geometry {
    static constexpr int TX = 32 * CX;         // tile width in cells
    static constexpr int W = TX + 8;           // E/H row: 4 cells of halo each side (TMA wants 16 B)
    static constexpr int WM = TX + 32;         // index row: 16 cells each side
    static constexpr int ER = kTileY + 2;      // E rows: y0-1 .. y0+TY
    static constexpr int HR = kTileY + 1;      // H rows: y0-1 .. y0+TY-1
    static constexpr int E_BYTES = 3 * ER * W * 4;
    static constexpr int H_BYTES = 3 * HR * W * 4;
    static constexpr int M_BYTES = HR * WM;
    static constexpr int align(int v) { return (v + 127) & ~127; }
    static constexpr int E_OFF = 0;
    static constexpr int H_OFF = align(E_BYTES);
    static constexpr int M_OFF = H_OFF + align(H_BYTES);
    static constexpr int SLOT = M_OFF + align(M_BYTES);
    static constexpr int TX_BYTES = E_BYTES + H_BYTES + M_BYTES; // bytes TMA lands per slot
    static constexpr int COEFF_OFF = kSlots * SLOT;
    static constexpr int BAR_OFF = COEFF_OFF + kMaxMaterials * 16;
    static constexpr int SMEM = BAR_OFF + kSlots * 8;
};

struct FusedArgs {
    DeviceScene s;
    float *e_out;
    float *h_out;
    float *intensity;       // null: not accumulating
    int32_t *error;         // set when a wait gives up
    uint32_t tiles_x, tiles_y, z_chunk;
    InjectionTable inj;
};

// ---- PTX wrappers -----------------------------------------------------------

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint32_t bar, uint32_t parity) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    return done != 0;
}

// Waits for a phase of an mbarrier, but never forever.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long budget) {
    const long long start = clock64();
    while (!mbar_try_wait(bar, parity))
        if (clock64() - start > budget) return false;
    return true;
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, int c,
                                            uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
        ::"r"(dst), "l"(map), "r"(x), "r"(y), "r"(z), "r"(c), "r"(bar)
        : "memory");
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, int x, int y, int z, uint32_t bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
        ::"r"(dst), "l"(map), "r"(x), "r"(y), "r"(z), "r"(bar)
        : "memory");
}

// ---- small vector helpers ---------------------------------------------------

template <int CX> struct Vec { float v[CX]; };

template <int CX> __device__ __forceinline__ Vec<CX> lds(const float *p) {
    Vec<CX> r;
    if constexpr (CX == 4) {
        float4 t = *reinterpret_cast<const float4 *>(p);
        r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    } else if constexpr (CX == 2) {
        float2 t = *reinterpret_cast<const float2 *>(p);
        r.v[0] = t.x; r.v[1] = t.y;
    } else {
        r.v[0] = *p;
    }
    return r;
}

template <int CX> __device__ __forceinline__ void sts(float *p, const Vec<CX> &r) {
    if constexpr (CX == 4) *reinterpret_cast<float4 *>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
    else if constexpr (CX == 2) *reinterpret_cast<float2 *>(p) = make_float2(r.v[0], r.v[1]);
    else *p = r.v[0];
}

template <int CX> __device__ __forceinline__ Vec<CX> ldg(const float *p) {
    Vec<CX> r;
    if constexpr (CX == 4) {
        float4 t = __ldg(reinterpret_cast<const float4 *>(p));
        r.v[0] = t.x; r.v[1] = t.y; r.v[2] = t.z; r.v[3] = t.w;
    } else if constexpr (CX == 2) {
        float2 t = __ldg(reinterpret_cast<const float2 *>(p));
        r.v[0] = t.x; r.v[1] = t.y;
    } else {
        r.v[0] = __ldg(p);
    }
    return r;
}

template <int CX> __device__ __forceinline__ void stg(float *p, const Vec<CX> &r) {
    if constexpr (CX == 4) __stcs(reinterpret_cast<float4 *>(p), make_float4(r.v[0], r.v[1], r.v[2], r.v[3]));
    else if constexpr (CX == 2) __stcs(reinterpret_cast<float2 *>(p), make_float2(r.v[0], r.v[1]));
    else __stcs(p, r.v[0]);
}

// Profile or gain samples for CX consecutive cells along x; cells past the
// end of the axis read as zero (they are never stored).  Scalar loads: the
// sections of the packed tables need not be 16-byte aligned, and this runs
// once per CTA.
template <int CX> __device__ __forceinline__ Vec<CX> ldg_x(const float *base, int x, int nx) {
    Vec<CX> r;
#pragma unroll
    for (int j = 0; j < CX; ++j) r.v[j] = (x + j >= 0 && x + j < nx) ? __ldg(base + x + j) : 0.0f;
    return r;
}

__device__ __forceinline__ float ldg_at(const float *base, int i, int n) {
    return (i >= 0 && i < n) ? __ldg(base + i) : 0.0f;
}

// The reference's semi-implicit updates (src/material.rs:131-146).  A zero
// total loss reduces ((1-l)v ± g·c)/(1+l) to v ± g·c exactly.
__device__ __forceinline__ float h_update(float h, float loss, float gain, float curl) {
    if (loss == 0.0f) return h - gain * curl;
    return ((1.0f - loss) * h - gain * curl) / (1.0f + loss);
}

__device__ __forceinline__ float e_update(float e, float loss, float gain, float curl) {
    if (loss == 0.0f) return e + gain * curl;
    return ((1.0f - loss) * e + gain * curl) / (1.0f + loss);
}

// Adds every injection of one phase that targets (component, cell) in the
// order the host listed them, which is the reference's order.
__device__ __forceinline__ float inject(const InjectionTable &t, const DeviceScene &s, bool magnetic,
                                        uint32_t component, int x, int y, int z, float value) {
    for (uint32_t k = 0; k < t.count; ++k) {
        const DeviceInjection &d = t.item[k];
        if (d.magnetic != uint32_t(magnetic) || d.component != component) continue;
        const int dx = x - int(d.origin[0]), dy = y - int(d.origin[1]), dz = z - int(d.origin[2]);
        if (dx < 0 || dy < 0 || dz < 0 || dx >= int(d.extent[0]) || dy >= int(d.extent[1]) || dz >= int(d.extent[2]))
            continue;
        const float weight = d.weight_offset < 0
                                 ? 1.0f
                                 : __ldg(&s.weights[d.weight_offset + (uint64_t(dz) * d.extent[1] + dy) * d.extent[0] + dx]);
        value += d.value * weight;
    }
    return value;
}

// Does any injection of this phase touch plane z / row y at all?
__device__ __forceinline__ bool touches(const InjectionTable &t, bool magnetic, int y, int z) {
    for (uint32_t k = 0; k < t.count; ++k) {
        const DeviceInjection &d = t.item[k];
        if (d.magnetic == uint32_t(magnetic) && z >= int(d.origin[2]) && z < int(d.origin[2] + d.extent[2]) &&
            y >= int(d.origin[1]) && y < int(d.origin[1] + d.extent[1]))
            return true;
    }
    return false;
}

template <int CX>
__global__ void __launch_bounds__(kThreads, 2)
fused_step(const __grid_constant__ CUtensorMap e_map, const __grid_constant__ CUtensorMap h_map,
           const __grid_constant__ CUtensorMap m_map, const __grid_constant__ FusedArgs args) {
    using G = Geometry<CX>;
    extern __shared__ __align__(128) unsigned char smem[];
    const DeviceScene &s = args.s;
    const int nx = int(s.n[0]), ny = int(s.n[1]), nz = int(s.n[2]);
    const uint64_t cells = s.cells;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const uint32_t tile = blockIdx.x % (args.tiles_x * args.tiles_y);
    const uint32_t chunk = blockIdx.x / (args.tiles_x * args.tiles_y);
    const int x0 = int(tile % args.tiles_x) * G::TX;
    const int y0 = int(tile / args.tiles_x) * kTileY;
    const int z0 = int(chunk * args.z_chunk);
    const int z1 = min(z0 + int(args.z_chunk), nz);
    // A chunk that does not start at the bottom first rebuilds new H one
    // plane below itself: E(z0) needs it.
    const int zs = z0 > 0 ? z0 - 1 : z0;

    float4 *coeff = reinterpret_cast<float4 *>(smem + G::COEFF_OFF);
    const uint32_t bar0 = smem_addr(smem + G::BAR_OFF);

    for (int m = threadIdx.x; m < kMaxMaterials; m += kThreads) coeff[m] = __ldg(&s.coeff[m]);
    if (threadIdx.x == 0) {
        for (int k = 0; k < kSlots; ++k) mbar_init(bar0 + 8 * k, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    // Plane p goes to slot (p - zs) % kSlots; its n-th use of that slot is
    // phase n & 1.
    auto issue = [&](int p) {
        const int k = (p - zs) % kSlots;
        unsigned char *slot = smem + k * G::SLOT;
        const uint32_t bar = bar0 + 8 * k;
        mbar_expect_tx(bar, G::TX_BYTES);
        tma_load_4d(smem_addr(slot + G::E_OFF), &e_map, x0 - 4, y0 - 1, p, 0, bar);
        tma_load_4d(smem_addr(slot + G::H_OFF), &h_map, x0 - 4, y0 - 1, p, 0, bar);
        tma_load_3d(smem_addr(slot + G::M_OFF), &m_map, x0 - 16, y0 - 1, p, bar);
    };
    const int last_plane = z1; // E(z1) feeds H(z1-1); past nz it arrives as zeros
    if (threadIdx.x == 0)
        for (int p = zs; p <= min(zs + kSlots - 1, last_plane); ++p) issue(p);

    // Per-thread constants: this lane's cells along x, this warp's row.
    const bool halo = warp == kTileY;
    const int row = halo ? 0 : warp + 1;     // row in the H slot (and E slot)
    const int y = y0 + row - 1;
    const int xl = x0 + CX * lane;           // first cell of this lane
    const int col = 4 + CX * lane;           // its column in an E/H slot row
    const int mcol = 16 + CX * lane;         // its column in an index slot row
    const uint32_t span = s.n[0] + s.n[1] + s.n[2];
    const float *absorb_int = s.absorber;
    const float *absorb_half = s.absorber + span;
    const Vec<CX> mgx = ldg_x<CX>(s.mgain, xl, nx), egx = ldg_x<CX>(s.egain, xl, nx);
    const Vec<CX> aix = ldg_x<CX>(absorb_int, xl, nx), ahx = ldg_x<CX>(absorb_half, xl, nx);
    const float mgy = ldg_at(s.mgain + nx, y, ny), egy = ldg_at(s.egain + nx, y, ny);
    const float aiy = ldg_at(absorb_int + nx, y, ny), ahy = ldg_at(absorb_half + nx, y, ny);
    // The halo column (x0-1) is handled by halo-warp lanes 0..TY-1, one row each.
    const int hy_row = lane + 1, hy_y = y0 + lane;
    const float hc_mgx = ldg_at(s.mgain, x0 - 1, nx);
    const float hc_ahx = ldg_at(absorb_half, x0 - 1, nx);
    const float hc_mgy = ldg_at(s.mgain + nx, hy_y, ny);
    const float hc_aiy = ldg_at(absorb_int + nx, hy_y, ny), hc_ahy = ldg_at(absorb_half + nx, hy_y, ny);
    const bool store_row = !halo && y < ny && xl < nx;

    Vec<CX> hx_prev, hy_prev; // new H at plane z-1, this thread's cells
#pragma unroll
    for (int j = 0; j < CX; ++j) hx_prev.v[j] = hy_prev.v[j] = 0.0f;

    for (int p = zs; p < z1; ++p) {
        const int k = (p - zs) % kSlots, k1 = (p + 1 - zs) % kSlots;
        const uint32_t phase = uint32_t((p - zs) / kSlots) & 1u, phase1 = uint32_t((p + 1 - zs) / kSlots) & 1u;
        bool ok = true;
        if (p == zs) ok = mbar_wait_bounded(bar0 + 8 * k, phase, kWaitCycles);
        ok = ok && mbar_wait_bounded(bar0 + 8 * k1, phase1, kWaitCycles);
        if (__syncthreads_or(!ok)) {
            // Give up on this chunk: report, then let the loads already in
            // flight land before the CTA's shared memory goes away.
            if (threadIdx.x == 0) {
                atomicExch(args.error, 1);
                for (int q = p; q <= min(p + kSlots - 1, last_plane); ++q) {
                    const int kq = (q - zs) % kSlots;
                    mbar_wait_bounded(bar0 + 8 * kq, uint32_t((q - zs) / kSlots) & 1u, kWaitCycles);
                }
            }
            __syncthreads();
            return;
        }
        // The slot plane p-1 used is free again: refill it two planes ahead.
        if (threadIdx.x == 0 && p > zs && p - 1 + kSlots <= last_plane) {
            asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
            issue(p - 1 + kSlots);
        }

        const float *E = reinterpret_cast<const float *>(smem + k * G::SLOT + G::E_OFF);
        const float *E1 = reinterpret_cast<const float *>(smem + k1 * G::SLOT + G::E_OFF);
        float *H = reinterpret_cast<float *>(smem + k * G::SLOT + G::H_OFF);
        const uint8_t *M = smem + k * G::SLOT + G::M_OFF;
        auto e_at = [&](const float *base, int c, int r, int cc) { return base + (c * G::ER + r) * G::W + cc; };
        auto h_at = [&](float *base, int c, int r, int cc) { return base + (c * G::HR + r) * G::W + cc; };

        const bool prologue = p < z0;
        const float mgz = __ldg(&s.mgain[nx + ny + p]), egz = __ldg(&s.egain[nx + ny + p]);
        const float aiz = __ldg(&absorb_int[nx + ny + p]), ahz = __ldg(&absorb_half[nx + ny + p]);
        const uint64_t plane_base = uint64_t(p) * ny * nx;

        // Intensity of this thread's cells, fetched early.
        Vec<CX> inten;
        const bool accumulate = args.intensity != nullptr && !prologue && store_row;
        if (accumulate) inten = ldg<CX>(args.intensity + plane_base + uint64_t(y) * nx + xl);

        // ---------------- H(p) ----------------
        if (!halo) {
            const Vec<CX> ex = lds<CX>(e_at(E, 0, row, col)), ex_up = lds<CX>(e_at(E, 0, row + 1, col));
            const Vec<CX> ey = lds<CX>(e_at(E, 1, row, col)), ez = lds<CX>(e_at(E, 2, row, col));
            const Vec<CX> ez_up = lds<CX>(e_at(E, 2, row + 1, col));
            const Vec<CX> ex_next = lds<CX>(e_at(E1, 0, row, col)), ey_next = lds<CX>(e_at(E1, 1, row, col));
            float ey_right = __shfl_down_sync(0xffffffffu, ey.v[0], 1);
            float ez_right = __shfl_down_sync(0xffffffffu, ez.v[0], 1);
            if (lane == 31) {
                ey_right = *e_at(E, 1, row, col + CX);
                ez_right = *e_at(E, 2, row, col + CX);
            }
            const Vec<CX> hx = lds<CX>(h_at(H, 0, row, col)), hy = lds<CX>(h_at(H, 1, row, col));
            const Vec<CX> hz = lds<CX>(h_at(H, 2, row, col));
            const float row_x = ahy + ahz, row_y = aiy + ahz, row_z = ahy + aiz;
            Vec<CX> nhx, nhy, nhz;
#pragma unroll
            for (int j = 0; j < CX; ++j) {
                const float4 c = coeff[M[row * G::WM + mcol + j]];
                const float eyr = j + 1 < CX ? ey.v[j + 1] : ey_right;
                const float ezr = j + 1 < CX ? ez.v[j + 1] : ez_right;
                const float curl_x = mgy * (ez_up.v[j] - ez.v[j]) - mgz * (ey_next.v[j] - ey.v[j]);
                const float curl_y = mgz * (ex_next.v[j] - ex.v[j]) - mgx.v[j] * (ezr - ez.v[j]);
                const float curl_z = mgx.v[j] * (eyr - ey.v[j]) - mgy * (ex_up.v[j] - ex.v[j]);
                nhx.v[j] = h_update(hx.v[j], (c.w + row_x) + aix.v[j], c.z, curl_x);
                nhy.v[j] = h_update(hy.v[j], (c.w + row_y) + ahx.v[j], c.z, curl_y);
                nhz.v[j] = h_update(hz.v[j], (c.w + row_z) + ahx.v[j], c.z, curl_z);
            }
            if (args.inj.count && touches(args.inj, true, y, p)) {
#pragma unroll
                for (int j = 0; j < CX; ++j) {
                    nhx.v[j] = inject(args.inj, s, true, 0, xl + j, y, p, nhx.v[j]);
                    nhy.v[j] = inject(args.inj, s, true, 1, xl + j, y, p, nhy.v[j]);
                    nhz.v[j] = inject(args.inj, s, true, 2, xl + j, y, p, nhz.v[j]);
                }
            }
            if (prologue) {
                hx_prev = nhx;
                hy_prev = nhy;
            } else {
                sts<CX>(h_at(H, 0, row, col), nhx);
                sts<CX>(h_at(H, 1, row, col), nhy);
                sts<CX>(h_at(H, 2, row, col), nhz);
                if (store_row) {
                    const uint64_t at = plane_base + uint64_t(y) * nx + xl;
                    stg<CX>(args.h_out + at, nhx);
                    stg<CX>(args.h_out + cells + at, nhy);
                    stg<CX>(args.h_out + 2 * cells + at, nhz);
                }
            }
        } else if (!prologue) {
            // Halo row y0-1: the Hx and Hz that E at row y0 reads.
            {
                const int hr = 0, yy = y0 - 1;
                const float hmgy = ldg_at(s.mgain + nx, yy, ny);
                const float haiy = ldg_at(absorb_int + nx, yy, ny), hahy = ldg_at(absorb_half + nx, yy, ny);
                const Vec<CX> ex = lds<CX>(e_at(E, 0, hr, col)), ex_up = lds<CX>(e_at(E, 0, hr + 1, col));
                const Vec<CX> ey = lds<CX>(e_at(E, 1, hr, col)), ez = lds<CX>(e_at(E, 2, hr, col));
                const Vec<CX> ez_up = lds<CX>(e_at(E, 2, hr + 1, col));
                const Vec<CX> ey_next = lds<CX>(e_at(E1, 1, hr, col));
                float ey_right = __shfl_down_sync(0xffffffffu, ey.v[0], 1);
                if (lane == 31) ey_right = *e_at(E, 1, hr, col + CX);
                const Vec<CX> hx = lds<CX>(h_at(H, 0, hr, col)), hz = lds<CX>(h_at(H, 2, hr, col));
                const float row_x = hahy + ahz, row_z = hahy + aiz;
                (void)haiy;
                Vec<CX> nhx, nhz;
#pragma unroll
                for (int j = 0; j < CX; ++j) {
                    const float4 c = coeff[M[hr * G::WM + mcol + j]];
                    const float eyr = j + 1 < CX ? ey.v[j + 1] : ey_right;
                    const float curl_x = hmgy * (ez_up.v[j] - ez.v[j]) - mgz * (ey_next.v[j] - ey.v[j]);
                    const float curl_z = mgx.v[j] * (eyr - ey.v[j]) - hmgy * (ex_up.v[j] - ex.v[j]);
                    nhx.v[j] = h_update(hx.v[j], (c.w + row_x) + aix.v[j], c.z, curl_x);
                    nhz.v[j] = h_update(hz.v[j], (c.w + row_z) + ahx.v[j], c.z, curl_z);
                }
                if (args.inj.count && touches(args.inj, true, yy, p)) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nhx.v[j] = inject(args.inj, s, true, 0, xl + j, yy, p, nhx.v[j]);
                        nhz.v[j] = inject(args.inj, s, true, 2, xl + j, yy, p, nhz.v[j]);
                    }
                }
                sts<CX>(h_at(H, 0, hr, col), nhx);
                sts<CX>(h_at(H, 2, hr, col), nhz);
            }
            // Halo column x0-1, rows y0..y0+TY-1: the Hy and Hz that E at
            // column x0 reads.
            if (lane < kTileY) {
                const int hr = hy_row, xx = x0 - 1, cc = 3;
                const float ex = *e_at(E, 0, hr, cc), ex_up = *e_at(E, 0, hr + 1, cc);
                const float ey = *e_at(E, 1, hr, cc), ez = *e_at(E, 2, hr, cc);
                const float ex_next = *e_at(E1, 0, hr, cc);
                const float eyr = *e_at(E, 1, hr, cc + 1), ezr = *e_at(E, 2, hr, cc + 1);
                const float hy = *h_at(H, 1, hr, cc), hz = *h_at(H, 2, hr, cc);
                const float4 c = coeff[M[hr * G::WM + 15]];
                const float aix_h = ldg_at(absorb_int, xx, nx);
                (void)aix_h;
                const float curl_y = mgz * (ex_next - ex) - hc_mgx * (ezr - ez);
                const float curl_z = hc_mgx * (eyr - ey) - hc_mgy * (ex_up - ex);
                float nhy = h_update(hy, (c.w + (hc_aiy + ahz)) + hc_ahx, c.z, curl_y);
                float nhz = h_update(hz, (c.w + (hc_ahy + aiz)) + hc_ahx, c.z, curl_z);
                if (args.inj.count) {
                    nhy = inject(args.inj, s, true, 1, xx, hy_y, p, nhy);
                    nhz = inject(args.inj, s, true, 2, xx, hy_y, p, nhz);
                }
                *h_at(H, 1, hr, cc) = nhy;
                *h_at(H, 2, hr, cc) = nhz;
            }
        }
        if (prologue) continue; // CTA-uniform: nobody wrote shared memory
        __syncthreads();

        // ---------------- E(p) ----------------
        if (!halo) {
            const Vec<CX> hx = lds<CX>(h_at(H, 0, row, col)), hy = lds<CX>(h_at(H, 1, row, col));
            const Vec<CX> hz = lds<CX>(h_at(H, 2, row, col));
            const Vec<CX> hx_dn = lds<CX>(h_at(H, 0, row - 1, col)), hz_dn = lds<CX>(h_at(H, 2, row - 1, col));
            float hy_left = __shfl_up_sync(0xffffffffu, hy.v[CX - 1], 1);
            float hz_left = __shfl_up_sync(0xffffffffu, hz.v[CX - 1], 1);
            if (lane == 0) {
                hy_left = *h_at(H, 1, row, col - 1);
                hz_left = *h_at(H, 2, row, col - 1);
            }
            Vec<CX> ex = lds<CX>(e_at(E, 0, row, col)), ey = lds<CX>(e_at(E, 1, row, col));
            Vec<CX> ez = lds<CX>(e_at(E, 2, row, col));
            const float row_x = aiy + aiz, row_y = ahy + aiz, row_z = aiy + ahz;
#pragma unroll
            for (int j = 0; j < CX; ++j) {
                const int x = xl + j;
                const float4 c = coeff[M[row * G::WM + mcol + j]];
                const float hyl = j > 0 ? hy.v[j - 1] : hy_left;
                const float hzl = j > 0 ? hz.v[j - 1] : hz_left;
                if (y != 0 && p != 0) {
                    const float curl = egy * (hz.v[j] - hz_dn.v[j]) - egz * (hy.v[j] - hy_prev.v[j]);
                    ex.v[j] = e_update(ex.v[j], (c.y + row_x) + ahx.v[j], c.x, curl);
                }
                if (p != 0 && x != 0) {
                    const float curl = egz * (hx.v[j] - hx_prev.v[j]) - egx.v[j] * (hz.v[j] - hzl);
                    ey.v[j] = e_update(ey.v[j], (c.y + row_y) + aix.v[j], c.x, curl);
                }
                if (x != 0 && y != 0) {
                    const float curl = egx.v[j] * (hy.v[j] - hyl) - egy * (hx.v[j] - hx_dn.v[j]);
                    ez.v[j] = e_update(ez.v[j], (c.y + row_z) + aix.v[j], c.x, curl);
                }
            }
            if (args.inj.count && touches(args.inj, false, y, p)) {
#pragma unroll
                for (int j = 0; j < CX; ++j) {
                    ex.v[j] = inject(args.inj, s, false, 0, xl + j, y, p, ex.v[j]);
                    ey.v[j] = inject(args.inj, s, false, 1, xl + j, y, p, ey.v[j]);
                    ez.v[j] = inject(args.inj, s, false, 2, xl + j, y, p, ez.v[j]);
                }
            }
            if (store_row) {
                const uint64_t at = plane_base + uint64_t(y) * nx + xl;
                stg<CX>(args.e_out + at, ex);
                stg<CX>(args.e_out + cells + at, ey);
                stg<CX>(args.e_out + 2 * cells + at, ez);
                if (accumulate) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        float sum = ex.v[j] * ex.v[j];
                        sum += ey.v[j] * ey.v[j];
                        sum += ez.v[j] * ez.v[j];
                        inten.v[j] += sum;
                    }
                    stg<CX>(args.intensity + at, inten);
                }
            }
            hx_prev = hx;
            hy_prev = hy;
        }
    }
    // Drain: every issued plane has been waited for (the loop waits through
    // plane z1, the last one issued), so no copy is still landing here.
}

// ---- host side ----------------------------------------------------------------

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPoint("cuTensorMapEncodeTiled", &p, cudaEnableDefault, &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess || p == nullptr)
            return EncodeTiled(nullptr);
        return reinterpret_cast<EncodeTiled>(p);
    }();
    return fn;
}

void encode(CUtensorMap *map, CUtensorMapDataType type, int rank, void *base, const cuuint64_t *dims,
            const cuuint64_t *strides, const cuuint32_t *box) {
    EncodeTiled fn = encoder();
    if (!fn) throw std::runtime_error("cuTensorMapEncodeTiled is unavailable");
    cuuint32_t elem[4] = {1, 1, 1, 1};
    CUresult r = fn(map, type, cuuint32_t(rank), base, dims, strides, box, elem, CU_TENSOR_MAP_INTERLEAVE_NONE,
                    CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
                    CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw std::runtime_error("cuTensorMapEncodeTiled failed: " + std::to_string(int(r)));
}

template <int CX> void configure() {
    static bool done = false;
    if (done) return;
    cudaFuncSetAttribute(fused_step<CX>, cudaFuncAttributeMaxDynamicSharedMemorySize, Geometry<CX>::SMEM);
    done = true;
}

int pick_cx(uint32_t nx) {
    // The widest tile that wastes no more lanes than a narrower one.
    int best = 4;
    uint32_t best_waste = ~0u;
    for (int cx : {4, 2, 1}) {
        uint32_t tx = 32u * cx, tiles = (nx + tx - 1) / tx, waste = tiles * tx - nx;
        if (waste < best_waste) {
            best = cx;
            best_waste = waste;
        }
    }
    return best;
}

} // namespace

bool fused_supported(const uint32_t n[3]) {
    // TMA needs 16-byte row strides for the f32 fields.
    return n[0] % 4 == 0 && n[0] >= 4 && n[1] >= 2 && n[2] >= 2 && encoder() != nullptr;
}

FusedPlan fused_plan(const uint32_t n[3], uint32_t tile_y, uint32_t z_chunk, int sm_count) {
    (void)tile_y;
    FusedPlan p{};
    p.tile_y = kTileY;
    p.cx = pick_cx(n[0]);
    const uint32_t tx = 32u * p.cx;
    p.tiles_x = (n[0] + tx - 1) / tx;
    p.tiles_y = (n[1] + kTileY - 1) / kTileY;
    const uint32_t tiles = p.tiles_x * p.tiles_y;
    if (z_chunk == 0) {
        // Enough chunks that the grid fills a few waves of two CTAs per SM,
        // but no thinner than 16 planes (each chunk rebuilds one extra plane).
        const uint32_t slots = 2u * uint32_t(sm_count > 0 ? sm_count : 1);
        uint32_t chunks = (4 * slots + tiles - 1) / tiles;
        chunks = chunks < 1 ? 1 : chunks;
        z_chunk = (n[2] + chunks - 1) / chunks;
        if (z_chunk < 16) z_chunk = 16;
    }
    p.z_chunk = z_chunk > n[2] ? n[2] : z_chunk;
    p.chunks = (n[2] + p.z_chunk - 1) / p.z_chunk;
    p.grid = tiles * p.chunks;
    p.smem = p.cx == 4 ? Geometry<4>::SMEM : (p.cx == 2 ? Geometry<2>::SMEM : Geometry<1>::SMEM);
    return p;
}

void fused_maps(const DeviceScene &s, const FusedPlan &plan, FieldSet set, const uint8_t *material_padded,
                uint32_t material_pitch, FusedMaps &out) {
    const uint32_t tx = 32u * plan.cx;
    const cuuint64_t nx = s.n[0], ny = s.n[1], nz = s.n[2];
    {
        cuuint64_t dims[4] = {nx, ny, nz, 3};
        cuuint64_t strides[3] = {nx * 4, nx * ny * 4, nx * ny * nz * 4};
        cuuint32_t ebox[4] = {tx + 8, kTileY + 2, 1, 3};
        cuuint32_t hbox[4] = {tx + 8, kTileY + 1, 1, 3};
        encode(reinterpret_cast<CUtensorMap *>(out.e), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, set.e, dims, strides, ebox);
        encode(reinterpret_cast<CUtensorMap *>(out.h), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, set.h, dims, strides, hbox);
    }
    {
        cuuint64_t dims[3] = {material_pitch, ny, nz};
        cuuint64_t strides[2] = {material_pitch, cuuint64_t(material_pitch) * ny};
        cuuint32_t box[3] = {tx + 32, kTileY + 1, 1};
        encode(reinterpret_cast<CUtensorMap *>(out.m), CU_TENSOR_MAP_DATA_TYPE_UINT8, 3,
               const_cast<uint8_t *>(material_padded), dims, strides, box);
    }
}

void launch_fused_step(const DeviceScene &s, const FusedPlan &plan, const FusedMaps &in_maps, FieldSet out,
                       float *intensity, const InjectionTable &table, int32_t *error, cudaStream_t stream) {
    FusedArgs args{};
    args.s = s;
    args.e_out = out.e;
    args.h_out = out.h;
    args.intensity = intensity;
    args.error = error;
    args.tiles_x = plan.tiles_x;
    args.tiles_y = plan.tiles_y;
    args.z_chunk = plan.z_chunk;
    args.inj = table;
    const CUtensorMap &em = *reinterpret_cast<const CUtensorMap *>(in_maps.e);
    const CUtensorMap &hm = *reinterpret_cast<const CUtensorMap *>(in_maps.h);
    const CUtensorMap &mm = *reinterpret_cast<const CUtensorMap *>(in_maps.m);
    switch (plan.cx) {
    case 4:
        configure<4>();
        fused_step<4><<<plan.grid, kThreads, plan.smem, stream>>>(em, hm, mm, args);
        break;
    case 2:
        configure<2>();
        fused_step<2><<<plan.grid, kThreads, plan.smem, stream>>>(em, hm, mm, args);
        break;
    default:
        configure<1>();
        fused_step<1><<<plan.grid, kThreads, plan.smem, stream>>>(em, hm, mm, args);
        break;
    }
}

} // namespace diaphane
