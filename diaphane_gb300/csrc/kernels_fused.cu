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
//     one cell outside the tile, so the CTA recomputes H there from the same
//     inputs instead of waiting for the neighbouring CTA (the TX + TY halo
//     cells are packed one per lane onto the first warps, so the other warps
//     skip that step).
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
// A warp in which only a few lanes hold lossy cells (the absorber edge or a
// lossy slab crossing a tile row) hands their divisions to all 32 lanes
// through a small per-warp scratch instead of letting every lane divide.
// Sources are applied to each freshly computed value in the reference's
// order (src/cpu.rs:606-633), halo cells included, and intensity is summed
// from the final E (src/cpu.rs:186-196).  The result is bit-identical to the
// reference's two-pass f32 step.
#include "device.cuh"
#include "exact_div.cuh"

#include <cuda.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <stdexcept>
#include <string>

namespace diaphane {

namespace {

constexpr int kMaxMaterials = 256;
constexpr long long kWaitCycles = 1ll << 32; // ~2 s at 2 GHz, then give up

// The budget of the plane waits, in clock cycles: kWaitCycles, unless a test
// lowers it to show the give-up path on the device (0 gives up at the first
// plane).  The drain after a give-up always keeps the full bound, so every
// load a CTA issued lands before it exits.
__device__ long long g_ring_wait_budget = kWaitCycles;

// CX cells per lane along x, TY rows per tile (one warp each), SLOTS planes
// in the shared-memory ring.
template <int CX, int TY, int SLOTS> struct Geometry {
    static constexpr int kWarps = TY;
    static constexpr int kThreads = 32 * TY;
    static constexpr int kSlots = SLOTS;
    static constexpr int TX = 32 * CX;         // tile width in cells
    static constexpr int W = TX + 8;           // E/H row: 4 cells of halo each side (TMA wants 16 B)
    static constexpr int WM = TX + 32;         // index row: 16 cells each side
    static constexpr int ER = TY + 2;          // E rows: y0-1 .. y0+TY
    static constexpr int HR = TY + 1;          // H rows: y0-1 .. y0+TY-1
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
    // Per warp: numerators and denominators of a compacted division: at most
    // three division rounds on the 128-wide tile, two on the 64-wide and one
    // on the 32-wide (on the narrow tiles a deeper compaction measured 0.3-
    // 0.4 % slower on the mixed batch than dividing in place).
    static constexpr int kCompactItems = CX == 4 ? 96 : (CX == 2 ? 64 : 32);
    static constexpr int SCRATCH_OFF = (BAR_OFF + kSlots * 8 + 15) & ~15;
    static constexpr int SCRATCH_WARP = 2 * kCompactItems * 4;
    static constexpr int INJ_OFF = SCRATCH_OFF + kWarps * SCRATCH_WARP; // 16-aligned
    static constexpr int SMEM = INJ_OFF + kMaxInjections * int(sizeof(DeviceInjection));
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
// The clock is read only once the first probe finds the phase incomplete,
// so a plane that has already landed costs one try_wait.  A budget of 0 or
// less gives up without probing.
__device__ __forceinline__ bool mbar_wait_bounded(uint32_t bar, uint32_t parity, long long budget) {
    if (budget <= 0) return false;
    if (mbar_try_wait(bar, parity)) return true;
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

// Stores CX cells, or only the first `valid` of them at the end of a row.
template <int CX> __device__ __forceinline__ void stg_row(float *p, const Vec<CX> &r, int valid) {
    if (valid >= CX) {
        stg<CX>(p, r);
        return;
    }
#pragma unroll
    for (int j = 0; j < CX; ++j)
        if (j < valid) __stcs(p + j, r.v[j]);
}

// The three components of a field at one lane's cells, one test of the row
// end for all three.
template <int CX>
__device__ __forceinline__ void stg_row3(float *p, uint64_t stride, const Vec<CX> &a, const Vec<CX> &b,
                                         const Vec<CX> &c, int valid) {
    if (valid >= CX) {
        stg<CX>(p, a);
        stg<CX>(p + stride, b);
        stg<CX>(p + 2 * stride, c);
        return;
    }
#pragma unroll
    for (int j = 0; j < CX; ++j)
        if (j < valid) {
            __stcs(p + j, a.v[j]);
            __stcs(p + stride + j, b.v[j]);
            __stcs(p + 2 * stride + j, c.v[j]);
        }
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

// The reference's semi-implicit updates (src/material.rs:131-146), in full.
// With a total loss of exactly zero they reduce to v ∓ g·c bit for bit, which
// is what the fast path below computes; either form is exact for l = 0.
__device__ __forceinline__ float h_full(float h, float loss, float gain, float curl) {
    return exact_div((1.0f - loss) * h - gain * curl, 1.0f + loss);
}

// Axis orders.  A batch may store a scene with its axes permuted, so that the
// axis that fills tile rows best runs along x (a 40 x 100 x 150-cell scene
// wastes fewer lanes as 150 x 100 x 40): stored axis i holds the scene's axis
// kBatchAxisOrders[order][i].  The step then performs the scene's own
// operations on the same operands, so its results are the unpermuted run's
// bit for bit:
//  * the curl of component a is the difference term along a+1 minus the one
//    along a+2 (src/cpu.rs:323-325, 423-424); an odd permutation reverses the
//    cyclic order.  Such a scene's gain tables are stored negated: each term
//    t becomes -t, and (-t1) - (-t2) equals t2 - t1 exactly, signed zeros
//    included (x - y is x + (-y), and IEEE addition commutes);
//  * the loss is (material + (absorber_y + absorber_z)) + absorber_x in the
//    scene's axes (src/cpu.rs:326 with the row sum of
//    src/boundary.rs:186-196): the kernel adds its two axes that are not the
//    scene's x first (loss_of below; 32-wide tiles only, wider tiles being
//    given scenes whose x is stored along x);
//  * the intensity adds the squares of the scene's Ex and Ey, then Ez's
//    (src/cpu.rs:186-194).
// Nothing negates a field (a difference that cancels exactly is +0 in either
// frame, so negated fields would not be exact).

// The total loss of one cell component from the material's and the absorber
// samples along the stored x (`lane`), y (`row`) and z (`plane`), the sample
// along the scene's x (stored axis SCENE_X) added last.
template <int SCENE_X> __device__ __forceinline__ float loss_of(float k, float lane, float row, float plane) {
    if constexpr (SCENE_X == 0) return (k + (row + plane)) + lane;
    else if constexpr (SCENE_X == 1) return (k + (lane + plane)) + row;
    else return (k + (lane + row)) + plane;
}

// |E|² of one cell, the square of stored component `scene_z` (the scene's
// Ez) added last.
__device__ __forceinline__ float squares_of(float ex, float ey, float ez, uint32_t scene_z) {
    float sum;
    if (scene_z == 2) {
        sum = ex * ex;
        sum += ey * ey;
        sum += ez * ez;
    } else if (scene_z == 1) {
        sum = ex * ex;
        sum += ez * ez;
        sum += ey * ey;
    } else {
        sum = ey * ey;
        sum += ez * ez;
        sum += ex * ex;
    }
    return sum;
}

// The division step of a warp in which only a few lanes hold lossy cells.
// Those lanes put their 3·CX numerators and denominators in the warp's
// scratch, all 32 lanes divide them (one item each per round), and each lossy
// lane reads its quotients back: ceil(items / 32) divisions per lane instead
// of 3·CX.  A quotient is the same correctly rounded value whichever lane
// computes it.  The lossless lanes' numerators are already their results
// (their denominators are exactly 1).
template <int CX>
__device__ __forceinline__ void divide_compacted(float *scratch, int items_max, unsigned lossy_lanes, int lane,
                                                 bool lossy, Vec<CX> &n0, Vec<CX> &n1, Vec<CX> &n2,
                                                 const float (&l0)[CX], const float (&l1)[CX],
                                                 const float (&l2)[CX]) {
    constexpr int K = 3 * CX;
    float *num = scratch, *den = scratch + items_max;
    const int rank = __popc(lossy_lanes & ((1u << lane) - 1u));
    if (lossy) {
        Vec<CX> d0, d1, d2;
#pragma unroll
        for (int j = 0; j < CX; ++j) {
            d0.v[j] = 1.0f + l0[j];
            d1.v[j] = 1.0f + l1[j];
            d2.v[j] = 1.0f + l2[j];
        }
        float *n = num + rank * K, *d = den + rank * K;
        sts<CX>(n, n0);
        sts<CX>(n + CX, n1);
        sts<CX>(n + 2 * CX, n2);
        sts<CX>(d, d0);
        sts<CX>(d + CX, d1);
        sts<CX>(d + 2 * CX, d2);
    }
    __syncwarp();
    const int items = __popc(lossy_lanes) * K;
    for (int i = lane; i < items; i += 32) num[i] = exact_div(num[i], den[i]);
    __syncwarp();
    if (lossy) {
        const float *n = num + rank * K;
        n0 = lds<CX>(n);
        n1 = lds<CX>(n + CX);
        n2 = lds<CX>(n + 2 * CX);
    }
}

// Bit k is set when injection k of `magnetic` phase covers row y, any of the
// cells [xa, xb) and any of the planes [za, zb) the thread will compute.
// Computed once per thread; the per-plane test is then a single z comparison
// per set bit, and a one-plane face (a total-field box's) costs nothing to the
// units that do not reach its plane.
// The injections of one step as the kernel reads them: a table in kernel
// parameters (one scene) or in global memory (a batch).
struct InjectionView {
    const DeviceInjection *item;
    uint32_t count;
    const float *profiles; // total-field box profile values of the step, or null
};

__device__ __forceinline__ uint32_t injection_mask(const InjectionView &t, bool magnetic, int xa, int xb, int y,
                                                   int za, int zb) {
    uint32_t m = 0;
    for (uint32_t k = 0; k < t.count; ++k) {
        // (origin x, y, z, extent x), (extent y, z, component, magnetic)
        const int4 w0 = reinterpret_cast<const int4 *>(&t.item[k])[0];
        const int4 w1 = reinterpret_cast<const int4 *>(&t.item[k])[1];
        if (w1.w == int(magnetic) && y >= w0.y && y < w0.y + w1.x && xb > w0.x && xa < w0.x + w0.w &&
            zb > w0.z && za < w0.z + w1.y)
            m |= 1u << k;
    }
    return m;
}

// Adds the injections in `mask` to the CX cells starting at x, in table
// order — the reference's order (src/cpu.rs:606-633).
template <int CX>
__device__ __forceinline__ void apply_injections(const InjectionView &t, const float *weights, uint32_t mask, int x,
                                                 int y, int z, Vec<CX> &f0, Vec<CX> &f1, Vec<CX> &f2) {
    while (mask) {
        const int k = __ffs(mask) - 1;
        mask &= mask - 1;
        const DeviceInjection &d = t.item[k];
        // The descriptor as three 16-byte words: (origin x, y, z, extent x),
        // (extent y, z, component, magnetic), (value, weight and profile
        // offsets, profile axis).
        const int4 w0 = reinterpret_cast<const int4 *>(&d)[0];
        const int4 w1 = reinterpret_cast<const int4 *>(&d)[1];
        const int4 w2 = reinterpret_cast<const int4 *>(&d)[2];
        const int dz = z - w0.z;
        if (dz < 0 || dz >= w1.y) continue;
        const int dy = y - w0.y;
        if (w2.y < 0 && w2.z < 0) {
            // Weight 1 everywhere (a point, a plane, a box's uniform face):
            // value * 1 is value, so each covered cell just adds it.
            const int dx0 = x - w0.x;
            const uint32_t ex = uint32_t(w0.w);
            const float add = __int_as_float(w2.x);
            // The component is the injection's, the same on every lane: one
            // branch, then selects (not an added zero: -0 + 0 would turn a
            // cell's -0 into +0).
            if (w1.z == 0) {
#pragma unroll
                for (int j = 0; j < CX; ++j) f0.v[j] = uint32_t(dx0 + j) < ex ? f0.v[j] + add : f0.v[j];
            } else if (w1.z == 1) {
#pragma unroll
                for (int j = 0; j < CX; ++j) f1.v[j] = uint32_t(dx0 + j) < ex ? f1.v[j] + add : f1.v[j];
            } else {
#pragma unroll
                for (int j = 0; j < CX; ++j) f2.v[j] = uint32_t(dx0 + j) < ex ? f2.v[j] + add : f2.v[j];
            }
            continue;
        }
#pragma unroll
        for (int j = 0; j < CX; ++j) {
            const int dx = x + j - int(d.origin[0]);
            if (dx < 0 || dx >= int(d.extent[0])) continue;
            const float w = injection_weight<float>(d, weights, t.profiles, uint32_t(x + j), uint32_t(y), uint32_t(z),
                                                    (uint64_t(dz) * d.extent[1] + dy) * d.extent[0] + dx);
            const float add = d.value * w;
            if (d.component == 0) f0.v[j] += add;
            else if (d.component == 1) f1.v[j] += add;
            else f2.v[j] += add;
        }
    }
}

__device__ __forceinline__ void apply_injections_1(const InjectionView &t, const float *weights, uint32_t mask,
                                                   int x, int y, int z, float &f0, float &f1, float &f2) {
    Vec<1> a{{f0}}, b{{f1}}, c{{f2}};
    apply_injections<1>(t, weights, mask, x, y, z, a, b, c);
    f0 = a.v[0];
    f1 = b.v[0];
    f2 = c.v[0];
}

// CX material indices of one lane, from its slot row.
template <int CX> __device__ __forceinline__ void load_materials(const uint8_t *p, uint32_t out[CX]) {
    if constexpr (CX == 4) {
        const uint32_t w = *reinterpret_cast<const uint32_t *>(p);
#pragma unroll
        for (int j = 0; j < 4; ++j) out[j] = (w >> (8 * j)) & 0xffu;
    } else if constexpr (CX == 2) {
        const uint32_t w = *reinterpret_cast<const uint16_t *>(p);
        out[0] = w & 0xffu;
        out[1] = w >> 8;
    } else {
        out[0] = *p;
    }
}

// One H cell update of all three components from slot values: used for the
// halo cells, where each lane owns a single cell.
struct HaloCell {
    int hr, hc;                  // slot row and column
    float mgx, mgy, aix, ahx, aiy, ahy;
    uint32_t mask;               // magnetic injections covering the cell
    int x, y;
};

// What one CTA needs to advance one tile of one scene through a chunk of
// z-planes.
struct UnitArgs {
    DeviceScene s;
    float *e_out;
    float *h_out;
    float *intensity;       // null: not accumulating
    int32_t *error;         // set when a wait gives up
    InjectionView inj;
    int x0, y0, z0, z1;     // tile origin and planes [z0, z1)
    uint32_t scene_z = 2;   // stored axis holding the scene's z (batch scenes)
};

// The fused step for one (scene, tile, z-chunk) unit; every kernel below is
// this function applied to a unit chosen from its block index.
//
// SCENE_X: the stored axis holding the scene's x (0 but for batch scenes on
// 32-wide tiles).  ANY_ORDER: the scene may be stored in any axis order (the
// batch kernels), whose intensity order u.scene_z gives.
template <int CX, int TY, int SLOTS, int SCENE_X = 0, bool ANY_ORDER = false>
__device__ __forceinline__ void step_unit(const CUtensorMap *e_map_p, const CUtensorMap *h_map_p,
                                          const CUtensorMap *m_map_p, const UnitArgs &u) {
    using G = Geometry<CX, TY, SLOTS>;
    static_assert(SCENE_X == 0 || (ANY_ORDER && CX == 1), "scenes with x stored elsewhere run 32-wide");
    constexpr int kWarps = G::kWarps, kThreads = G::kThreads, kSlots = G::kSlots;
    extern __shared__ __align__(128) unsigned char smem[];
    const DeviceScene &s = u.s;
    // The step's injections, staged in shared memory below with the
    // coefficient table: the per-plane tests and additions read them there.
    DeviceInjection *inj_staged = reinterpret_cast<DeviceInjection *>(smem + G::INJ_OFF);
    const InjectionView inj{inj_staged, u.inj.count, u.inj.profiles};
    const int nx = int(s.n[0]), ny = int(s.n[1]);
    const uint64_t pitch = s.pitch;
    const uint64_t cells = s.cells;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int x0 = u.x0, y0 = u.y0, z0 = u.z0, z1 = u.z1;
    // A chunk that does not start at the bottom first rebuilds new H one
    // plane below itself: E(z0) needs it.
    const int zs = z0 > 0 ? z0 - 1 : z0;

    float4 *coeff = reinterpret_cast<float4 *>(smem + G::COEFF_OFF);
    const uint32_t bar0 = smem_addr(smem + G::BAR_OFF);

    // Plane p goes to slot (p - zs) % kSlots; its n-th use of that slot is
    // phase n & 1.
    auto issue = [&](int p) {
        const int k = (p - zs) % kSlots;
        unsigned char *slot = smem + k * G::SLOT;
        const uint32_t bar = bar0 + 8 * k;
        mbar_expect_tx(bar, G::TX_BYTES);
        tma_load_4d(smem_addr(slot + G::E_OFF), e_map_p, x0 - 4, y0 - 1, p, 0, bar);
        tma_load_4d(smem_addr(slot + G::H_OFF), h_map_p, x0 - 4, y0 - 1, p, 0, bar);
        tma_load_3d(smem_addr(slot + G::M_OFF), m_map_p, x0 - 16, y0 - 1, p, bar);
    };
    const int last_plane = z1; // E(z1) feeds H(z1-1); past nz it arrives as zeros
    // The first planes are requested before the coefficient table is staged,
    // so the two latencies overlap; the barrier below publishes both the
    // table and the initialised ring barriers.
    if (threadIdx.x == 0) {
        for (int k = 0; k < kSlots; ++k) mbar_init(bar0 + 8 * k, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int p = zs; p <= min(zs + kSlots - 1, last_plane); ++p) issue(p);
    }
    for (int m = threadIdx.x; m < kMaxMaterials; m += kThreads) coeff[m] = __ldg(&s.coeff[m]);
    {
        constexpr int kWords = int(sizeof(DeviceInjection) / 4);
        const uint32_t *from = reinterpret_cast<const uint32_t *>(u.inj.item);
        uint32_t *to = reinterpret_cast<uint32_t *>(inj_staged);
        const int words = int(u.inj.count) * kWords;
        for (int w = threadIdx.x; w < words; w += kThreads) to[w] = from[w];
    }
    __syncthreads();

    // Per-thread constants: this lane's cells along x, this warp's row.
    const int row = warp + 1;                // row in the E and H slots
    const int y = y0 + warp;
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
    const bool store_row = y < ny && xl < nx;
    // Cells at or past nx in this lane (only when the row pitch is wider than
    // the grid) are computed but never stored.
    const int full_lane = nx - xl >= CX ? CX : nx - xl;
    const bool has_inj = inj.count != 0;
    // Both phases' masks in one pass over the table.
    uint32_t mask_h = 0, mask_e = 0;
    for (uint32_t k = 0; k < inj.count; ++k) {
        // (origin x, y, z, extent x), (extent y, z, component, magnetic)
        const int4 w0 = reinterpret_cast<const int4 *>(&inj.item[k])[0];
        const int4 w1 = reinterpret_cast<const int4 *>(&inj.item[k])[1];
        if (y >= w0.y && y < w0.y + w1.x && xl + CX > w0.x && xl < w0.x + w0.w && z1 > w0.z && zs < w0.z + w1.y) {
            if (w1.w) mask_h |= 1u << k;
            else mask_e |= 1u << k;
        }
    }

    // Halo cells, packed onto the first warps: halo index i = 32·warp + lane;
    // i < TX takes cell x0+i of row y0-1 (the Hx, Hz that E at row y0 reads),
    // TX <= i < TX+TY takes cell (x0-1, y0+i-TX) (the Hy, Hz that E at x0
    // reads).  The remaining warps skip the halo step altogether.
    constexpr int kHalo = G::TX + kWarps;
    static_assert(kHalo <= kThreads, "every halo cell needs a thread");
    const int halo_index = 32 * warp + lane;
    const bool halo_lane = halo_index < kHalo;
    const int halo_in_warp = kHalo - 32 * warp; // > 0 on warps holding halo cells
    const unsigned halo_mask = halo_in_warp >= 32 ? 0xffffffffu : (halo_in_warp > 0 ? (1u << halo_in_warp) - 1u : 0u);
    HaloCell hc{};
    if (halo_lane) {
        if (halo_index < G::TX) {
            hc.hr = 0;
            hc.hc = 4 + halo_index;
            hc.x = x0 + halo_index;
            hc.y = y0 - 1;
        } else {
            hc.hr = halo_index - G::TX + 1;
            hc.hc = 3;
            hc.x = x0 - 1;
            hc.y = y0 + (halo_index - G::TX);
        }
        hc.mgx = ldg_at(s.mgain, hc.x, nx);
        hc.aix = ldg_at(absorb_int, hc.x, nx);
        hc.ahx = ldg_at(absorb_half, hc.x, nx);
        hc.mgy = ldg_at(s.mgain + nx, hc.y, ny);
        hc.aiy = ldg_at(absorb_int + nx, hc.y, ny);
        hc.ahy = ldg_at(absorb_half + nx, hc.y, ny);
        hc.mask = has_inj ? injection_mask(inj, true, hc.x, hc.x + 1, hc.y, zs, z1) : 0u;
    }

    float *scratch = reinterpret_cast<float *>(smem + G::SCRATCH_OFF + warp * G::SCRATCH_WARP);

    Vec<CX> hx_prev, hy_prev; // new H at plane z-1, this thread's cells
#pragma unroll
    for (int j = 0; j < CX; ++j) hx_prev.v[j] = hy_prev.v[j] = 0.0f;

    const long long ring_budget = g_ring_wait_budget;
    for (int p = zs; p < z1; ++p) {
        const int k = (p - zs) % kSlots, k1 = (p + 1 - zs) % kSlots;
        const uint32_t phase = uint32_t((p - zs) / kSlots) & 1u, phase1 = uint32_t((p + 1 - zs) / kSlots) & 1u;
        // Every thread waits on the ring itself: a lone poller followed by a
        // barrier measured ~30% slower (the barrier adds the poller's wake-up
        // latency to every plane).
        bool ok = ring_budget > 0;
        if (p == zs) ok = ok && mbar_wait_bounded(bar0 + 8 * k, phase, ring_budget);
        ok = ok && mbar_wait_bounded(bar0 + 8 * k1, phase1, ring_budget);
        if (__syncthreads_or(!ok)) {
            // Give up on this chunk: report, then let the loads already in
            // flight land before the CTA's shared memory goes away.
            // Issued so far: the first kSlots planes, then at each later plane
            // the one kSlots - 1 ahead of the one before (its refill comes below).
            if (threadIdx.x == 0) {
                atomicExch(u.error, 1);
                const int issued = min(p == zs ? zs + kSlots - 1 : p + kSlots - 2, last_plane);
                for (int q = p; q <= issued; ++q) {
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
        const uint64_t at = (uint64_t(p) * ny + uint64_t(y)) * pitch + xl; // this lane's first cell

        // Intensity of this thread's cells, fetched early.
        Vec<CX> inten;
        const bool accumulate = u.intensity != nullptr && !prologue && store_row;
        if (accumulate) inten = ldg<CX>(u.intensity + at);

        // Material coefficients of this lane's cells, kept for the E phase.
        float2 ecoef[CX]; // (electric_gain, electric_loss)

        // New H at this thread's cells, kept in registers for the E phase
        // (the other warps read it from the H slot).
        Vec<CX> kept_hx, kept_hy, kept_hz;
        // Old E at this thread's cells, kept from the H phase on the 32- and
        // 64-wide tiles (3 and 6 registers; the 128-wide tile reads it again
        // from the slot, its registers being spoken for).
        Vec<CX> kept_ex, kept_ey, kept_ez;
        // ---------------- H(p): this warp's row ----------------
        {
            const Vec<CX> ex = lds<CX>(e_at(E, 0, row, col)), ex_up = lds<CX>(e_at(E, 0, row + 1, col));
            const Vec<CX> ey = lds<CX>(e_at(E, 1, row, col)), ez = lds<CX>(e_at(E, 2, row, col));
            const Vec<CX> ez_up = lds<CX>(e_at(E, 2, row + 1, col));
            if constexpr (CX <= 2) {
                kept_ex = ex;
                kept_ey = ey;
                kept_ez = ez;
            }
            const Vec<CX> ex_next = lds<CX>(e_at(E1, 0, row, col)), ey_next = lds<CX>(e_at(E1, 1, row, col));
            // The right neighbour's first cell: the next lane's, except past
            // the last lane.  The narrow tiles read it from the slot (no
            // shuffle, no lane-31 branch: 1 % faster on the mixed batch); the
            // 128-wide tile shuffles (the slot reads cost it 4 %).
            float ey_right, ez_right;
            if constexpr (CX <= 2) {
                ey_right = *e_at(E, 1, row, col + CX);
                ez_right = *e_at(E, 2, row, col + CX);
            } else {
                ey_right = __shfl_down_sync(0xffffffffu, ey.v[0], 1);
                ez_right = __shfl_down_sync(0xffffffffu, ez.v[0], 1);
                if (lane == 31) {
                    ey_right = *e_at(E, 1, row, col + CX);
                    ez_right = *e_at(E, 2, row, col + CX);
                }
            }
            Vec<CX> nhx = lds<CX>(h_at(H, 0, row, col)), nhy = lds<CX>(h_at(H, 1, row, col));
            Vec<CX> nhz = lds<CX>(h_at(H, 2, row, col));
            uint32_t mat[CX];
            load_materials<CX>(M + row * G::WM + mcol, mat);
            const float row_x = ahy + ahz, row_y = aiy + ahz, row_z = ahy + aiz;
            float gain[CX], lx[CX], ly[CX], lz[CX], cx_[CX], cy_[CX], cz_[CX];
            bool lossless = true;
#pragma unroll
            for (int j = 0; j < CX; ++j) {
                const float4 c = coeff[mat[j]];
                ecoef[j] = make_float2(c.x, c.y);
                gain[j] = c.z;
                const float eyr = j + 1 < CX ? ey.v[j + 1] : ey_right;
                const float ezr = j + 1 < CX ? ez.v[j + 1] : ez_right;
                cx_[j] = mgy * (ez_up.v[j] - ez.v[j]) - mgz * (ey_next.v[j] - ey.v[j]);
                cy_[j] = mgz * (ex_next.v[j] - ex.v[j]) - mgx.v[j] * (ezr - ez.v[j]);
                cz_[j] = mgx.v[j] * (eyr - ey.v[j]) - mgy * (ex_up.v[j] - ex.v[j]);
                if constexpr (SCENE_X == 0) {
                    lx[j] = (c.w + row_x) + aix.v[j];
                    ly[j] = (c.w + row_y) + ahx.v[j];
                    lz[j] = (c.w + row_z) + ahx.v[j];
                } else {
                    lx[j] = loss_of<SCENE_X>(c.w, aix.v[j], ahy, ahz);
                    ly[j] = loss_of<SCENE_X>(c.w, ahx.v[j], aiy, ahz);
                    lz[j] = loss_of<SCENE_X>(c.w, ahx.v[j], ahy, aiz);
                }
                lossless = lossless && lx[j] == 0.0f && ly[j] == 0.0f && lz[j] == 0.0f;
            }
            const unsigned lossy_lanes = __ballot_sync(0xffffffffu, !lossless);
            if (lossy_lanes == 0) {
#pragma unroll
                for (int j = 0; j < CX; ++j) {
                    nhx.v[j] = nhx.v[j] - gain[j] * cx_[j];
                    nhy.v[j] = nhy.v[j] - gain[j] * cy_[j];
                    nhz.v[j] = nhz.v[j] - gain[j] * cz_[j];
                }
            } else {
                float n0[CX], n1[CX], n2[CX];
#pragma unroll
                for (int j = 0; j < CX; ++j) {
                    n0[j] = (1.0f - lx[j]) * nhx.v[j] - gain[j] * cx_[j];
                    n1[j] = (1.0f - ly[j]) * nhy.v[j] - gain[j] * cy_[j];
                    n2[j] = (1.0f - lz[j]) * nhz.v[j] - gain[j] * cz_[j];
                }
                // All numerators zero (a field the wave has not reached yet:
                // ±0 / d = ±0)?  One vote on each lane's first value settles
                // the common case, where the field is there.
                bool zero = false;
                if (__all_sync(0xffffffffu, n0[0] == 0.0f)) {
                    zero = true;
#pragma unroll
                    for (int j = 0; j < CX; ++j) zero = zero && n0[j] == 0.0f && n1[j] == 0.0f && n2[j] == 0.0f;
                    zero = __all_sync(0xffffffffu, zero);
                }
                if (zero) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nhx.v[j] = n0[j];
                        nhy.v[j] = n1[j];
                        nhz.v[j] = n2[j];
                    }
                } else if (__popc(lossy_lanes) * 3 * CX <= G::kCompactItems) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nhx.v[j] = n0[j];
                        nhy.v[j] = n1[j];
                        nhz.v[j] = n2[j];
                    }
                    divide_compacted<CX>(scratch, G::kCompactItems, lossy_lanes, lane, !lossless, nhx, nhy, nhz, lx,
                                         ly, lz);
                } else {
                    // Tested only here, where it is used: computed with the
                    // numerators for every lossy warp it cost 1.5 % of the
                    // 512³ step.
                    bool normal = true;
#pragma unroll
                    for (int j = 0; j < CX; ++j)
                        normal = normal && plain_division_is_fast(n0[j]) && plain_division_is_fast(n1[j]) &&
                                 plain_division_is_fast(n2[j]);
                    if (__all_sync(0xffffffffu, normal)) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nhx.v[j] = n0[j] / (1.0f + lx[j]);
                        nhy.v[j] = n1[j] / (1.0f + ly[j]);
                        nhz.v[j] = n2[j] / (1.0f + lz[j]);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nhx.v[j] = exact_div(n0[j], 1.0f + lx[j]);
                        nhy.v[j] = exact_div(n1[j], 1.0f + ly[j]);
                        nhz.v[j] = exact_div(n2[j], 1.0f + lz[j]);
                    }
                }
                }
            }
            if (mask_h) apply_injections<CX>(inj, s.weights, mask_h, xl, y, p, nhx, nhy, nhz);
            if (prologue) {
                hx_prev = nhx;
                hy_prev = nhy;
            } else {
                kept_hx = nhx;
                kept_hy = nhy;
                kept_hz = nhz;
                sts<CX>(h_at(H, 0, row, col), nhx);
                sts<CX>(h_at(H, 1, row, col), nhy);
                sts<CX>(h_at(H, 2, row, col), nhz);
                if (store_row) {
                    stg_row3<CX>(u.h_out + at, cells, nhx, nhy, nhz, full_lane);
                }
            }
        }
        if (prologue) continue; // CTA-uniform: nobody wrote shared memory

        // ---------------- H(p): halo cells ----------------
        if (halo_lane) {
            const int hr = hc.hr, cc = hc.hc;
            const float ex = *e_at(E, 0, hr, cc), ex_up = *e_at(E, 0, hr + 1, cc), ex_n = *e_at(E1, 0, hr, cc);
            const float ey = *e_at(E, 1, hr, cc), ey_r = *e_at(E, 1, hr, cc + 1), ey_n = *e_at(E1, 1, hr, cc);
            const float ez = *e_at(E, 2, hr, cc), ez_r = *e_at(E, 2, hr, cc + 1), ez_up = *e_at(E, 2, hr + 1, cc);
            const float4 c = coeff[M[hr * G::WM + cc + 12]];
            float nx_ = *h_at(H, 0, hr, cc), ny_ = *h_at(H, 1, hr, cc), nz_ = *h_at(H, 2, hr, cc);
            const float lx = loss_of<SCENE_X>(c.w, hc.aix, hc.ahy, ahz), ly = loss_of<SCENE_X>(c.w, hc.ahx, hc.aiy, ahz);
            const float lz = loss_of<SCENE_X>(c.w, hc.ahx, hc.ahy, aiz);
            const float cxh = hc.mgy * (ez_up - ez) - mgz * (ey_n - ey);
            const float cyh = mgz * (ex_n - ex) - hc.mgx * (ez_r - ez);
            const float czh = hc.mgx * (ey_r - ey) - hc.mgy * (ex_up - ex);
            if (__all_sync(halo_mask, lx == 0.0f && ly == 0.0f && lz == 0.0f)) {
                nx_ = nx_ - c.z * cxh;
                ny_ = ny_ - c.z * cyh;
                nz_ = nz_ - c.z * czh;
            } else {
                nx_ = h_full(nx_, lx, c.z, cxh);
                ny_ = h_full(ny_, ly, c.z, cyh);
                nz_ = h_full(nz_, lz, c.z, czh);
            }
            if (hc.mask) apply_injections_1(inj, s.weights, hc.mask, hc.x, hc.y, p, nx_, ny_, nz_);
            *h_at(H, 0, hr, cc) = nx_;
            *h_at(H, 1, hr, cc) = ny_;
            *h_at(H, 2, hr, cc) = nz_;
        }
        __syncthreads();

        // ---------------- E(p) ----------------
        {
            const Vec<CX> hx = kept_hx, hy = kept_hy, hz = kept_hz;
            const Vec<CX> hx_dn = lds<CX>(h_at(H, 0, row - 1, col)), hz_dn = lds<CX>(h_at(H, 2, row - 1, col));
            // The left neighbour's last new H (the halo column for lane 0):
            // from the slot on the narrow tiles, by shuffle on the wide one.
            float hy_left, hz_left;
            if constexpr (CX <= 2) {
                hy_left = *h_at(H, 1, row, col - 1);
                hz_left = *h_at(H, 2, row, col - 1);
            } else {
                hy_left = __shfl_up_sync(0xffffffffu, hy.v[CX - 1], 1);
                hz_left = __shfl_up_sync(0xffffffffu, hz.v[CX - 1], 1);
                if (lane == 0) {
                    hy_left = *h_at(H, 1, row, col - 1);
                    hz_left = *h_at(H, 2, row, col - 1);
                }
            }
            Vec<CX> ex, ey, ez;
            if constexpr (CX <= 2) {
                ex = kept_ex;
                ey = kept_ey;
                ez = kept_ez;
            } else {
                ex = lds<CX>(e_at(E, 0, row, col)), ey = lds<CX>(e_at(E, 1, row, col));
                ez = lds<CX>(e_at(E, 2, row, col));
            }
            const float row_x = aiy + aiz, row_y = ahy + aiz, row_z = aiy + ahz;
            float cx_[CX], cy_[CX], cz_[CX], lx[CX], ly[CX], lz[CX];
            bool lossless = true;
#pragma unroll
            for (int j = 0; j < CX; ++j) {
                const float hyl = j > 0 ? hy.v[j - 1] : hy_left;
                const float hzl = j > 0 ? hz.v[j - 1] : hz_left;
                cx_[j] = egy * (hz.v[j] - hz_dn.v[j]) - egz * (hy.v[j] - hy_prev.v[j]);
                cy_[j] = egz * (hx.v[j] - hx_prev.v[j]) - egx.v[j] * (hz.v[j] - hzl);
                cz_[j] = egx.v[j] * (hy.v[j] - hyl) - egy * (hx.v[j] - hx_dn.v[j]);
                if constexpr (SCENE_X == 0) {
                    lx[j] = (ecoef[j].y + row_x) + ahx.v[j];
                    ly[j] = (ecoef[j].y + row_y) + aix.v[j];
                    lz[j] = (ecoef[j].y + row_z) + aix.v[j];
                } else {
                    lx[j] = loss_of<SCENE_X>(ecoef[j].y, ahx.v[j], aiy, aiz);
                    ly[j] = loss_of<SCENE_X>(ecoef[j].y, aix.v[j], ahy, aiz);
                    lz[j] = loss_of<SCENE_X>(ecoef[j].y, aix.v[j], aiy, ahz);
                }
                lossless = lossless && lx[j] == 0.0f && ly[j] == 0.0f && lz[j] == 0.0f;
            }
            Vec<CX> nex, ney, nez;
            const unsigned lossy_lanes = __ballot_sync(0xffffffffu, !lossless);
            if (lossy_lanes == 0) {
#pragma unroll
                for (int j = 0; j < CX; ++j) {
                    nex.v[j] = ex.v[j] + ecoef[j].x * cx_[j];
                    ney.v[j] = ey.v[j] + ecoef[j].x * cy_[j];
                    nez.v[j] = ez.v[j] + ecoef[j].x * cz_[j];
                }
            } else {
                float n0[CX], n1[CX], n2[CX];
#pragma unroll
                for (int j = 0; j < CX; ++j) {
                    n0[j] = (1.0f - lx[j]) * ex.v[j] + ecoef[j].x * cx_[j];
                    n1[j] = (1.0f - ly[j]) * ey.v[j] + ecoef[j].x * cy_[j];
                    n2[j] = (1.0f - lz[j]) * ez.v[j] + ecoef[j].x * cz_[j];
                }
                // All numerators zero (a field the wave has not reached yet:
                // ±0 / d = ±0)?  One vote on each lane's first value settles
                // the common case, where the field is there.
                bool zero = false;
                if (__all_sync(0xffffffffu, n0[0] == 0.0f)) {
                    zero = true;
#pragma unroll
                    for (int j = 0; j < CX; ++j) zero = zero && n0[j] == 0.0f && n1[j] == 0.0f && n2[j] == 0.0f;
                    zero = __all_sync(0xffffffffu, zero);
                }
                if (zero) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nex.v[j] = n0[j];
                        ney.v[j] = n1[j];
                        nez.v[j] = n2[j];
                    }
                } else if (__popc(lossy_lanes) * 3 * CX <= G::kCompactItems) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nex.v[j] = n0[j];
                        ney.v[j] = n1[j];
                        nez.v[j] = n2[j];
                    }
                    divide_compacted<CX>(scratch, G::kCompactItems, lossy_lanes, lane, !lossless, nex, ney, nez, lx,
                                         ly, lz);
                } else {
                    bool normal = true;
#pragma unroll
                    for (int j = 0; j < CX; ++j)
                        normal = normal && plain_division_is_fast(n0[j]) && plain_division_is_fast(n1[j]) &&
                                 plain_division_is_fast(n2[j]);
                    if (__all_sync(0xffffffffu, normal)) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nex.v[j] = n0[j] / (1.0f + lx[j]);
                        ney.v[j] = n1[j] / (1.0f + ly[j]);
                        nez.v[j] = n2[j] / (1.0f + lz[j]);
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        nex.v[j] = exact_div(n0[j], 1.0f + lx[j]);
                        ney.v[j] = exact_div(n1[j], 1.0f + ly[j]);
                        nez.v[j] = exact_div(n2[j], 1.0f + lz[j]);
                    }
                }
                }
            }
            // Index 0 along b or c is never written: the low-wall conductor
            // (src/cpu.rs:386-394).
            const bool update_x = y != 0 && p != 0;
#pragma unroll
            for (int j = 0; j < CX; ++j) {
                const bool x_inner = xl + j != 0;
                ex.v[j] = update_x ? nex.v[j] : ex.v[j];
                ey.v[j] = (p != 0 && x_inner) ? ney.v[j] : ey.v[j];
                ez.v[j] = (x_inner && y != 0) ? nez.v[j] : ez.v[j];
            }
            if (mask_e) apply_injections<CX>(inj, s.weights, mask_e, xl, y, p, ex, ey, ez);
            if (store_row) {
                stg_row3<CX>(u.e_out + at, cells, ex, ey, ez, full_lane);
                if (accumulate) {
#pragma unroll
                    for (int j = 0; j < CX; ++j) {
                        if constexpr (ANY_ORDER) {
                            inten.v[j] += squares_of(ex.v[j], ey.v[j], ez.v[j], u.scene_z);
                        } else {
                            float sum = ex.v[j] * ex.v[j];
                            sum += ey.v[j] * ey.v[j];
                            sum += ez.v[j] * ez.v[j];
                            inten.v[j] += sum;
                        }
                    }
                    stg_row<CX>(u.intensity + at, inten, full_lane);
                }
            }
            hx_prev = hx;
            hy_prev = hy;
        }
    }
    // Every issued plane has been waited for (the loop waits through plane
    // z1, the last one issued), so no copy is still landing here.
}

// One scene: block b is tile b % tiles of z-chunk b / tiles.  Sixteen
// resident warps x 128 registers fill each SM sub-partition's 16K-register
// file exactly: two CTAs of 8 warps, or one of 16.
// CTAs per SM a kernel variant is built for.  Narrow tiles give each warp
// few cells per plane, so their fixed per-plane latency (ring waits,
// barriers, the division chain) is hidden only by more resident warps: the
// 64-wide form (3-slot ring, at most 80 registers) fits 3 CTAs per SM and the
// 32-wide form (4-slot ring, 64 registers) 4, measured 14 % faster on a batch
// of mixed small scenes than 2 CTAs of each.
constexpr int resident_ctas(int CX, int TY, int SLOTS) {
    return CX == 1 && SLOTS <= 4 ? 4 : (CX == 2 && SLOTS <= 3 ? 3 : 16 / TY);
}

template <int CX, int TY, int SLOTS>
__global__ void __launch_bounds__(32 * TY, resident_ctas(CX, TY, SLOTS))
fused_step(const __grid_constant__ CUtensorMap e_map, const __grid_constant__ CUtensorMap h_map,
           const __grid_constant__ CUtensorMap m_map, const __grid_constant__ FusedArgs args) {
    const uint32_t tiles = args.tiles_x * args.tiles_y;
    const uint32_t tile = blockIdx.x % tiles, chunk = blockIdx.x / tiles;
    UnitArgs u;
    u.s = args.s;
    u.e_out = args.e_out;
    u.h_out = args.h_out;
    u.intensity = args.intensity;
    u.error = args.error;
    u.inj = InjectionView{args.inj.item, args.inj.count, args.inj.profiles};
    u.x0 = int(tile % args.tiles_x) * 32 * CX;
    u.y0 = int(tile / args.tiles_x) * TY;
    u.z0 = int(chunk * args.z_chunk);
    u.z1 = min(u.z0 + int(args.z_chunk), int(args.s.n[2]));
    step_unit<CX, TY, SLOTS>(&e_map, &h_map, &m_map, u);
}

// A batch: block b is unit b of this variant's work list.  Scene descriptors
// (with their tensor maps) live in global memory; a scene that has finished
// its steps for this chunk, or has left the batch, is skipped.  Every scene
// of the list has its x stored along axis SCENE_X.
template <int CX, int TY, int SLOTS, int SCENE_X>
__global__ void __launch_bounds__(32 * TY, resident_ctas(CX, TY, SLOTS))
fused_batch_step(const BatchScene *__restrict__ scenes, const BatchUnit *__restrict__ units,
                 const DeviceInjection *__restrict__ injections, const uint32_t *__restrict__ injection_counts,
                 const float *__restrict__ profiles, uint32_t scene_count, uint32_t step, int32_t *error) {
    const BatchUnit unit = units[blockIdx.x];
    const BatchScene &bs = scenes[unit.scene];
    if (step >= bs.steps) return;
    const uint32_t p = (bs.parity + step) & 1u;
    const CUtensorMap *e_map = reinterpret_cast<const CUtensorMap *>(bs.e_map[p]);
    const CUtensorMap *h_map = reinterpret_cast<const CUtensorMap *>(bs.h_map[p]);
    const CUtensorMap *m_map = reinterpret_cast<const CUtensorMap *>(bs.m_map);
    if (threadIdx.x == 0) {
        // The descriptors were written by a host copy since the last launch.
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(e_map) : "memory");
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(h_map) : "memory");
        asm volatile("fence.proxy.tensormap::generic.acquire.gpu [%0], 128;" ::"l"(m_map) : "memory");
    }
    UnitArgs u;
    u.s = bs.s;
    u.e_out = bs.e[p ^ 1u];
    u.h_out = bs.h[p ^ 1u];
    u.intensity = bs.intensity;
    u.error = error;
    const size_t slot = size_t(step) * scene_count + unit.scene;
    u.inj = InjectionView{injections + slot * kBatchInjections, injection_counts[slot], profiles};
    u.x0 = int(unit.x0);
    u.y0 = int(unit.y0);
    u.z0 = int(unit.z0);
    u.z1 = int(unit.z1);
    u.scene_z = bs.scene_z;
    step_unit<CX, TY, SLOTS, SCENE_X, true>(e_map, h_map, m_map, u);
}

// ---- host side ----------------------------------------------------------------

using EncodeTiled = CUresult (*)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                 const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encoder() {
    static EncodeTiled fn = [] {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        // The entry point as introduced in CUDA 12.0.
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
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

// A kernel's shared-memory opt-in is an attribute of the current device's
// context, so it is set once per device (a bit per device ordinal; host
// threads may race to set it, which is harmless).
template <int CX, int TY, int SLOTS> void configure() {
    static std::atomic<uint64_t> done{0};
    int device = 0;
    cudaGetDevice(&device);
    const uint64_t bit = device < 64 ? uint64_t(1) << device : 0;
    if (bit && (done.load(std::memory_order_acquire) & bit)) return;
    cudaFuncSetAttribute(fused_step<CX, TY, SLOTS>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         Geometry<CX, TY, SLOTS>::SMEM);
    cudaFuncSetAttribute(fused_step<CX, TY, SLOTS>, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    done.fetch_or(bit, std::memory_order_release);
}

template <int CX, int TY, int SLOTS> size_t smem_of() { return Geometry<CX, TY, SLOTS>::SMEM; }

size_t variant_smem(uint32_t cx, uint32_t ty, uint32_t slots) {
    if (cx == 4 && ty == 8 && slots == 3) return smem_of<4, 8, 3>();
    if (cx == 2 && ty == 8 && slots == 3) return smem_of<2, 8, 3>();
    if (cx == 2 && ty == 8 && slots == 5) return smem_of<2, 8, 5>();
    if (cx == 4 && ty == 16 && slots == 3) return smem_of<4, 16, 3>();
    if (cx == 1 && ty == 8 && slots == 4) return smem_of<1, 8, 4>();
    if (cx == 1 && ty == 8 && slots == 5) return smem_of<1, 8, 5>();
    return 0;
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

template <int CX, int TY, int SLOTS>
void launch_variant(const FusedPlan &plan, const FusedMaps &m, const FusedArgs &args, cudaStream_t stream) {
    configure<CX, TY, SLOTS>();
    fused_step<CX, TY, SLOTS><<<plan.grid, 32 * TY, plan.smem, stream>>>(
        *reinterpret_cast<const CUtensorMap *>(m.e), *reinterpret_cast<const CUtensorMap *>(m.h),
        *reinterpret_cast<const CUtensorMap *>(m.m), args);
}

} // namespace

bool fused_variant_exists(uint32_t cx, uint32_t ty, uint32_t slots) { return variant_smem(cx, ty, slots) != 0; }

FusedPlan fused_plan(const uint32_t n[3], uint32_t cx, uint32_t tile_y, uint32_t slots, uint32_t z_chunk,
                     int sm_count) {
    FusedPlan p{};
    p.cx = cx ? cx : uint32_t(pick_cx(n[0]));
    p.tile_y = tile_y ? tile_y : 8;
    const uint32_t tx = 32u * p.cx;
    p.tiles_x = (n[0] + tx - 1) / tx;
    p.tiles_y = (n[1] + p.tile_y - 1) / p.tile_y;
    const uint32_t tiles = p.tiles_x * p.tiles_y;
    if (slots == 0) {
        // The 64- and 32-wide tiles come in two builds: 3 or 4 CTAs per SM
        // (shallow ring, fewer registers) for grids that fill the GPU, and 2
        // CTAs per SM (5-slot ring, no register cap) for grids too small to
        // give every SM that many CTAs even in 16-plane chunks, where each
        // CTA's own latency is what counts.
        p.slots = p.cx == 1 && p.tile_y == 8 ? 4 : 3;
        if ((p.cx == 1 || p.cx == 2) && p.tile_y == 8) {
            const uint64_t shallow = uint64_t(tiles) * ((n[2] + 15) / 16);
            const uint64_t slots_on_gpu =
                uint64_t(resident_ctas(int(p.cx), 8, int(p.slots))) * uint64_t(sm_count > 0 ? sm_count : 1);
            if (shallow < slots_on_gpu) p.slots = 5;
        }
    } else {
        p.slots = slots;
    }
    p.smem = variant_smem(p.cx, p.tile_y, p.slots);
    if (p.smem == 0) throw std::runtime_error("no fused kernel variant with that tile shape and ring depth");
    p.ctas_per_sm = uint32_t(resident_ctas(int(p.cx), int(p.tile_y), int(p.slots)));
    if (z_chunk == 0) {
        // Pick the chunk depth whose CTA count fills whole waves best, among
        // depths of 16 to 32 planes (each chunk rebuilds one extra plane).
        // Deeper chunks measured slower even where they fill the waves as
        // well: at 384³ one wave of 192-plane chunks ran 0.829 ms a step
        // against 0.644-0.670 ms for 20- to 32-plane chunks, reading 18 %
        // more from DRAM (CTAs that walk far drift apart along z, and the
        // halo rows a neighbour shares no longer meet in L2).
        const uint32_t resident = p.ctas_per_sm * uint32_t(sm_count > 0 ? sm_count : 1);
        double best = 1e30;
        z_chunk = n[2];
        for (uint32_t depth = 16; depth <= std::min<uint32_t>(n[2] + 15, 32); ++depth) {
            const uint32_t chunks = (n[2] + depth - 1) / depth;
            const uint32_t waves = (tiles * chunks + resident - 1) / resident;
            const double cost = double(waves) * double(depth + 1);
            if (cost < best - 1e-9) {
                best = cost;
                z_chunk = depth;
            }
            if (depth >= n[2]) break;
        }
    }
    p.z_chunk = z_chunk > n[2] ? n[2] : z_chunk;
    p.chunks = (n[2] + p.z_chunk - 1) / p.z_chunk;
    p.grid = tiles * p.chunks;
    return p;
}

namespace {

// Field maps: the grid's true extent with the arena's row pitch, so reads past
// nx arrive as zeros (the wall) whatever the padding holds.
void encode_field_maps(const DeviceScene &s, uint32_t tx, uint32_t ty, float *e, float *h, void *e_out,
                       void *h_out) {
    const cuuint64_t nx = s.n[0], ny = s.n[1], nz = s.n[2], pitch = s.pitch;
    cuuint64_t dims[4] = {nx, ny, nz, 3};
    cuuint64_t strides[3] = {pitch * 4, pitch * ny * 4, pitch * ny * nz * 4};
    cuuint32_t ebox[4] = {tx + 8, ty + 2, 1, 3};
    cuuint32_t hbox[4] = {tx + 8, ty + 1, 1, 3};
    encode(reinterpret_cast<CUtensorMap *>(e_out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, e, dims, strides, ebox);
    encode(reinterpret_cast<CUtensorMap *>(h_out), CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, h, dims, strides, hbox);
}

void encode_index_map(const DeviceScene &s, uint32_t tx, uint32_t ty, const uint8_t *material,
                      uint32_t material_pitch, void *out) {
    const cuuint64_t ny = s.n[1], nz = s.n[2];
    cuuint64_t dims[3] = {material_pitch, ny, nz};
    cuuint64_t strides[2] = {material_pitch, cuuint64_t(material_pitch) * ny};
    cuuint32_t box[3] = {tx + 32, ty + 1, 1};
    encode(reinterpret_cast<CUtensorMap *>(out), CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, const_cast<uint8_t *>(material),
           dims, strides, box);
}

} // namespace

void fused_maps(const DeviceScene &s, const FusedPlan &plan, FieldSet set, const uint8_t *material_padded,
                uint32_t material_pitch, FusedMaps &out) {
    const uint32_t tx = 32u * plan.cx, ty = plan.tile_y;
    encode_field_maps(s, tx, ty, set.e, set.h, out.e, out.h);
    encode_index_map(s, tx, ty, material_padded, material_pitch, out.m);
}

void batch_scene_maps(BatchScene &scene, uint32_t cx, uint32_t tile_y, const uint8_t *material,
                      uint32_t material_pitch) {
    const uint32_t tx = 32u * cx;
    for (int k = 0; k < 2; ++k) encode_field_maps(scene.s, tx, tile_y, scene.e[k], scene.h[k], scene.e_map[k], scene.h_map[k]);
    encode_index_map(scene.s, tx, tile_y, material, material_pitch, scene.m_map);
}

size_t fused_variant_smem(uint32_t cx, uint32_t tile_y, uint32_t slots) { return variant_smem(cx, tile_y, slots); }

namespace {

template <int CX, int TY, int SLOTS, int SCENE_X> void configure_batch_variant() {
    cudaFuncSetAttribute(fused_batch_step<CX, TY, SLOTS, SCENE_X>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         Geometry<CX, TY, SLOTS>::SMEM);
    cudaFuncSetAttribute(fused_batch_step<CX, TY, SLOTS, SCENE_X>, cudaFuncAttributePreferredSharedMemoryCarveout,
                         100);
}

template <int CX, int TY, int SLOTS, int SCENE_X>
void launch_batch_variant(const BatchScene *scenes, const BatchUnit *units, uint32_t unit_count,
                          const DeviceInjection *injections, const uint32_t *counts, const float *profiles,
                          uint32_t scene_count, uint32_t step, int32_t *error, cudaStream_t stream) {
    fused_batch_step<CX, TY, SLOTS, SCENE_X><<<unit_count, 32 * TY, Geometry<CX, TY, SLOTS>::SMEM, stream>>>(
        scenes, units, injections, counts, profiles, scene_count, step, error);
}

} // namespace

void configure_batch_kernels() {
    configure_batch_variant<4, 8, 3, 0>();
    configure_batch_variant<2, 8, 3, 0>();
    configure_batch_variant<1, 8, 4, 0>();
    configure_batch_variant<1, 8, 4, 1>();
    configure_batch_variant<1, 8, 4, 2>();
}

bool tensor_maps_available() { return encoder() != nullptr; }

void set_ring_wait_budget(long long cycles) {
    const long long budget = cycles < 0 ? kWaitCycles : cycles;
    const cudaError_t err = cudaMemcpyToSymbol(g_ring_wait_budget, &budget, sizeof(budget));
    if (err != cudaSuccess) {
        cudaGetLastError();
        throw std::runtime_error(std::string("setting the ring wait budget: ") + cudaGetErrorString(err));
    }
}

void launch_batch_step(uint32_t cx, uint32_t tile_y, uint32_t slots, uint32_t scene_x, const BatchScene *scenes,
                       const BatchUnit *units, uint32_t unit_count, const DeviceInjection *injections,
                       const uint32_t *injection_counts, const float *profiles, uint32_t scene_count,
                       uint32_t step, int32_t *error, cudaStream_t stream) {
    if (unit_count == 0) return;
    if (cx == 4 && tile_y == 8 && slots == 3 && scene_x == 0)
        launch_batch_variant<4, 8, 3, 0>(scenes, units, unit_count, injections, injection_counts, profiles, scene_count, step, error, stream);
    else if (cx == 2 && tile_y == 8 && slots == 3 && scene_x == 0)
        launch_batch_variant<2, 8, 3, 0>(scenes, units, unit_count, injections, injection_counts, profiles, scene_count, step, error, stream);
    else if (cx == 1 && tile_y == 8 && slots == 4 && scene_x == 0)
        launch_batch_variant<1, 8, 4, 0>(scenes, units, unit_count, injections, injection_counts, profiles, scene_count, step, error, stream);
    else if (cx == 1 && tile_y == 8 && slots == 4 && scene_x == 1)
        launch_batch_variant<1, 8, 4, 1>(scenes, units, unit_count, injections, injection_counts, profiles, scene_count, step, error, stream);
    else if (cx == 1 && tile_y == 8 && slots == 4 && scene_x == 2)
        launch_batch_variant<1, 8, 4, 2>(scenes, units, unit_count, injections, injection_counts, profiles, scene_count, step, error, stream);
    else
        throw std::runtime_error("no batch kernel variant with that tile shape and ring depth");
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
    if (plan.cx == 4 && plan.tile_y == 8 && plan.slots == 3) launch_variant<4, 8, 3>(plan, in_maps, args, stream);
    else if (plan.cx == 2 && plan.tile_y == 8 && plan.slots == 3) launch_variant<2, 8, 3>(plan, in_maps, args, stream);
    else if (plan.cx == 4 && plan.tile_y == 16 && plan.slots == 3) launch_variant<4, 16, 3>(plan, in_maps, args, stream);
    else if (plan.cx == 1 && plan.tile_y == 8 && plan.slots == 4) launch_variant<1, 8, 4>(plan, in_maps, args, stream);
    else if (plan.cx == 2 && plan.tile_y == 8 && plan.slots == 5) launch_variant<2, 8, 5>(plan, in_maps, args, stream);
    else if (plan.cx == 1 && plan.tile_y == 8 && plan.slots == 5) launch_variant<1, 8, 5>(plan, in_maps, args, stream);
    else throw std::runtime_error("no fused kernel variant with that tile shape and ring depth");
}

} // namespace diaphane
