// Device-side view of a resolved scene and the launchers shared by the
// simulation host code (sim.cu) and the kernel translation units.
//
// Every kernel in this library is compiled with -fmad=false and IEEE
// division: the update expressions are evaluated in the reference's order with
// no multiply-add contraction, so a cell update is bit-identical to the
// reference's f32 arithmetic (src/cpu.rs:283-434).
#pragma once

#include <chrono>
#include <cstdint>
#include <thread>
#include <cuda_runtime.h>

namespace diaphane {

// Waits for a stream with a deadline: cudaSuccess when its work is done,
// cudaErrorNotReady when `timeout_ms` passed first, or the stream's error.
// The first 200 µs poll without sleeping, so a short wait (a field read, the
// end of a chunk) returns within a few µs of the work; longer waits poll
// every 50 µs.
inline cudaError_t poll_stream(cudaStream_t stream, uint32_t timeout_ms) {
    const auto start = std::chrono::steady_clock::now();
    const auto spin = start + std::chrono::microseconds(200);
    const auto deadline = start + std::chrono::milliseconds(timeout_ms);
    for (;;) {
        const cudaError_t q = cudaStreamQuery(stream);
        if (q != cudaErrorNotReady) return q;
        const auto now = std::chrono::steady_clock::now();
        if (now >= deadline) return cudaErrorNotReady;
        if (now >= spin) std::this_thread::sleep_for(std::chrono::microseconds(50));
    }
}

// Tables a step kernel reads.  All pointers are device pointers.
struct DeviceScene {
    uint32_t n[3];
    uint32_t pitch;          // row stride in cells (nx, or nx rounded up to 4 in a batch arena)
    uint64_t cells;          // component stride: pitch * ny * nz
    const uint8_t *material; // cells, u8 index (scenes of up to 256 materials)
    const uint16_t *material16; // cells, u16 index (wider scenes; material is null then)
    const float4 *coeff;     // (electric_gain, electric_loss, magnetic_gain, magnetic_loss)
    const float *mgain;      // nx | ny | nz, c*dt/primary width
    const float *egain;      // nx | ny | nz, c*dt/dual width
    const float *absorber;   // integer x|y|z, then half x|y|z
    const float *weights;    // sheet apodization planes
};

// The material of cell i, whichever width the index has.
__device__ __forceinline__ uint32_t material_of(const DeviceScene &s, uint64_t i) {
    return s.material16 ? uint32_t(s.material16[i]) : uint32_t(s.material[i]);
}

// One injection of one step (Injection, src/source.rs:409-427).
// 16-byte aligned so the step reads it as three 16-byte words.
struct alignas(16) DeviceInjection {
    uint32_t origin[3];
    uint32_t extent[3];
    uint32_t component;
    uint32_t magnetic;
    float value;
    int32_t weight_offset; // -1: weight 1
    // A total-field box's side face: the cell's weight is the step's
    // profile value at profile_offset + (coordinate - origin) along
    // profile_axis; -1: none.
    int32_t profile_offset;
    uint32_t profile_axis;
};
static_assert(sizeof(DeviceInjection) == 48, "three 16-byte words");

// Non-silent injections of one step, in the reference's application order.
constexpr int kMaxInjections = 32;
struct InjectionTable {
    uint32_t count;
    const float *profiles; // the step's box profile values (device), or null
    DeviceInjection item[kMaxInjections];
};

// The weight of cell (x, y, z) of injection d (d's box contains the cell).
template <typename T>
__device__ __forceinline__ T injection_weight(const DeviceInjection &d, const float *weights, const T *profiles,
                                              uint32_t x, uint32_t y, uint32_t z, uint64_t index_in_box) {
    if (d.profile_offset >= 0 && profiles != nullptr) {
        const uint32_t c = d.profile_axis == 0 ? x : (d.profile_axis == 1 ? y : z);
        return profiles[d.profile_offset + int32_t(c - d.origin[d.profile_axis])];
    }
    return d.weight_offset < 0 ? T(1) : T(__ldg(&weights[d.weight_offset + index_in_box]));
}

// Fields of one buffer set: component a of E at e + a*cells.  The step runs
// in float; the FP64 instance keeps its fields in double.
template <typename T> struct Fields {
    T *e;
    T *h;
};
using FieldSet = Fields<float>;
using FieldSet64 = Fields<double>;

// Naive path (kernels_naive.cu): one thread per cell, separate passes, in
// float or (the FP64 instance) double.
void launch_naive_magnetic(const DeviceScene &s, FieldSet f, bool reverse, cudaStream_t stream);
void launch_naive_magnetic(const DeviceScene &s, FieldSet64 f, bool reverse, cudaStream_t stream);
void launch_naive_electric(const DeviceScene &s, FieldSet f, bool reverse, cudaStream_t stream);
void launch_naive_electric(const DeviceScene &s, FieldSet64 f, bool reverse, cudaStream_t stream);
// `profiles`: the step's box profile values (device) when inj has one.
void launch_inject(const DeviceScene &s, FieldSet f, const DeviceInjection &inj, float sign, const float *profiles,
                   cudaStream_t stream);
// `value` is the signed drive in double; inj.value is not read.
void launch_inject(const DeviceScene &s, FieldSet64 f, const DeviceInjection &inj, double value,
                   const double *profiles, cudaStream_t stream);
void launch_intensity(const DeviceScene &s, const float *e, float *intensity, cudaStream_t stream);

// Dense <-> pitched rows of `components` fields of `rows` rows each (pitch.cu).
void launch_pack_rows(const float *src, float *dst, uint32_t nx, uint32_t pitch, uint64_t rows, uint64_t src_stride,
                      uint32_t components, cudaStream_t stream);
void launch_unpack_rows(const float *src, float *dst, uint32_t nx, uint32_t pitch, uint64_t rows, uint64_t dst_stride,
                        uint32_t components, cudaStream_t stream);

// Copies `components` pitched device fields (component stride `stride`) to or
// from dense host rows: one contiguous transfer, packed on the device when the
// pitch differs from nx.  Asynchronous on `stream`.
void copy_fields_out(float *host, const float *device, const uint32_t n[3], uint32_t pitch, uint64_t stride,
                     int components, cudaStream_t stream);
void copy_fields_in(float *device, const float *host, const uint32_t n[3], uint32_t pitch, uint64_t stride,
                    int components, cudaStream_t stream);

// Scene::material_indices on the device (raster.cu): the u8 index with rows of
// `pitch` bytes (padding cells 0), asynchronous on `stream`.
struct Scene;
void rasterize_on_device(const Scene &s, void *out, uint32_t pitch, cudaStream_t stream);

// Reductions (kernels_naive.cu).
void launch_energy(const DeviceScene &s, FieldSet f, const float *primary, const float *dual,
                   const float2 *eps_mu, double *partials, uint32_t blocks, cudaStream_t stream);
void launch_energy(const DeviceScene &s, FieldSet64 f, const float *primary, const float *dual,
                   const float2 *eps_mu, double *partials, uint32_t blocks, cudaStream_t stream);
void launch_finite(const DeviceScene &s, FieldSet f, int32_t *flag, cudaStream_t stream);
void launch_energy_density(const DeviceScene &s, FieldSet f, float *dense_out, cudaStream_t stream);
uint32_t energy_blocks(uint64_t cells);

// Fused path (kernels_fused.cu): one launch per step, reads one field set
// (through TMA tensor maps) and writes the other.
struct FusedPlan {
    uint32_t tile_y;      // rows per tile, one warp each
    uint32_t cx;          // cells per lane along x (tile width 32*cx)
    uint32_t slots;       // z-planes in the shared-memory ring
    uint32_t ctas_per_sm; // resident CTAs per SM the variant is sized for
    uint32_t z_chunk;     // planes per CTA
    uint32_t tiles_x, tiles_y, chunks;
    uint32_t grid;        // CTAs launched
    size_t smem;          // dynamic shared memory per CTA
};
// Plans dp_sim_autotune found fastest, per grid extent and device SM count,
// for the life of the process (tune.cu).  A simulation created for that
// shape with no plan options starts from it; a batch scene of that shape
// takes its tile width.
struct TunedPlan {
    uint32_t cx, tile_y, slots, z_chunk;
    float ms_per_step;
};
bool tuned_plan(const uint32_t n[3], int sms, TunedPlan &out);
void remember_tuned_plan(const uint32_t n[3], int sms, const TunedPlan &plan);

// Opaque 128-byte CUtensorMap images for one input field set.
struct FusedMaps {
    alignas(64) unsigned char e[128];
    alignas(64) unsigned char h[128];
    alignas(64) unsigned char m[128];
};
bool fused_variant_exists(uint32_t cx, uint32_t tile_y, uint32_t slots);
// Zero for cx, tile_y, slots or z_chunk picks the default.
FusedPlan fused_plan(const uint32_t n[3], uint32_t cx, uint32_t tile_y, uint32_t slots, uint32_t z_chunk,
                     int sm_count);
// material_padded: the u8 index with rows padded to material_pitch (a
// multiple of 16) so the tensor map's row stride is 16-byte aligned.
void fused_maps(const DeviceScene &s, const FusedPlan &plan, FieldSet set, const uint8_t *material_padded,
                uint32_t material_pitch, FusedMaps &out);
void launch_fused_step(const DeviceScene &s, const FusedPlan &plan, const FusedMaps &in_maps, FieldSet out,
                       float *intensity, const InjectionTable &table, int32_t *error, cudaStream_t stream);

// ---- batched form ------------------------------------------------------------

// Injections per scene per step in a batch (2 slots per source).
constexpr int kBatchInjections = 8;

// One scene of a batch, in global memory.  The three 128-byte CUtensorMap
// images come first so they keep the 64-byte alignment TMA requires.
struct alignas(64) BatchScene {
    unsigned char e_map[2][128];  // reading set 0 / set 1
    unsigned char h_map[2][128];
    unsigned char m_map[128];
    DeviceScene s;
    float *e[2];
    float *h[2];
    float *intensity;             // null: not accumulating
    uint32_t parity;              // set that holds the fields at the chunk's first step
    uint32_t steps;               // steps this scene takes in the chunk (0: idle)
    uint64_t step0;               // the scene's step count at the chunk's first step
    uint32_t scene_z;             // stored axis holding the scene's z (kBatchAxisOrders)
};

// One CTA's work: a tile of one scene through planes [z0, z1).
struct BatchUnit {
    uint32_t scene, x0, y0, z0, z1;
};

// Tensor maps of one batch scene (fields and index with row pitches).
void batch_scene_maps(BatchScene &scene, uint32_t cx, uint32_t tile_y, const uint8_t *material,
                      uint32_t material_pitch);
// Axis orders a batch scene can be stored in: stored axis i (x, y, z) holds
// the scene's axis kBatchAxisOrders[order][i].  Order 0 is the scene's own;
// 1-3 exchange two axes (a scene in one of these has its gain tables stored
// negated, which reverses every curl's subtraction), 4 and 5 rotate all
// three.  Scenes whose x is not stored along x run on 32-wide tiles.
constexpr int kBatchAxisOrders[6][3] = {{0, 1, 2}, {1, 0, 2}, {0, 2, 1}, {2, 1, 0}, {1, 2, 0}, {2, 0, 1}};

// One launch per step over every unit of one kernel variant: tile shape,
// ring depth, and the stored axis holding its scenes' x (1 and 2 for 32-wide
// tiles only).
// `profiles`: the chunk's total-field box profile values (device), which the
// injections' profile offsets index; null when no scene of the batch has a box.
void launch_batch_step(uint32_t cx, uint32_t tile_y, uint32_t slots, uint32_t scene_x, const BatchScene *scenes,
                       const BatchUnit *units, uint32_t unit_count, const DeviceInjection *injections,
                       const uint32_t *injection_counts, const float *profiles, uint32_t scene_count,
                       uint32_t step, int32_t *error, cudaStream_t stream);
size_t fused_variant_smem(uint32_t cx, uint32_t tile_y, uint32_t slots);
// Sets every batch kernel's shared-memory attributes (before any capture).
void configure_batch_kernels();
// Whether tensor maps can be encoded at all (driver entry point present).
bool tensor_maps_available();
// Test hook: the fused kernels' plane-wait budget on the current device, in
// clock cycles (negative: the default bound; 0: give up at the first plane).
void set_ring_wait_budget(long long cycles);

} // namespace diaphane
