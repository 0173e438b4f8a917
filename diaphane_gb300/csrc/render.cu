// Headless volume renderer for a live simulation: the reference viewer's
// volume pass (examples/common/shaders/volume.wgsl) and its host-side
// exposure control (examples/common/render.rs), as CUDA kernels writing an
// RGBA8 image into device memory instead of a swapchain.
//
// The ray-march reads the simulation's own field buffers — nothing is copied
// between the step kernel writing a field and the pixel that shows it — and
// samples a graded grid through a tabulated world-to-cell map
// (Grid::cell_lookup, src/grid.rs:635-646).  Per frame: the host folds the
// previous frame's peak reduction into a smoothed exposure (fast rise, slow
// fall, render.rs:281-325), the peak reduction runs again, and one thread per
// pixel marches the view ray.  Output is what the reference's sRGB capture
// target holds: the shaded linear colour, clamped and sRGB-encoded to 8 bits.
#include "sim.hpp"

#include <cfloat>
#include <cmath>

namespace {

constexpr int kPeakSlots = 8; // energy density peak, |E| and |H| per component, averaged intensity

enum : uint32_t {
    kModeEnergy = 0,
    kModeElectric = 1,
    kModeMagnetic = 2,
    kModeMagnitude = 3,
    kModeFields = 4,
    kModeGrid = 5,
    kModeRibbons = 6,
    kModeIntensity = 7,
};

struct V3 {
    float x, y, z;
};

__host__ __device__ inline float at(const V3 &v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// What the volume pass needs (ViewParams, render.rs:164-183).
struct ViewArgs {
    const float *e, *h, *intensity;
    uint64_t component_stride; // padded cells
    uint32_t n[3], pitch;
    const float *lookup;
    uint32_t samples;
    float box[3];
    float origin[3], march;
    float right[3], exposure;
    float up[3], log_strength;
    float forward[3];
    uint32_t mode;
    float inverse_path, played, window_start, bar_height;
    uint32_t component_e, component_h, accumulated;
    uint32_t width, height;
    uint8_t *image;
};

__device__ inline float mixf(float a, float b, float t) { return a * (1.0f - t) + b * t; }
__device__ inline V3 mix3(V3 a, V3 b, float t) { return V3{mixf(a.x, b.x, t), mixf(a.y, b.y, t), mixf(a.z, b.z, t)}; }
__device__ inline V3 add(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ inline V3 scale(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ inline V3 mul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
__device__ inline float signf(float v) { return v > 0.0f ? 1.0f : (v < 0.0f ? -1.0f : 0.0f); }
__device__ inline float clamp01(float v) { return fminf(fmaxf(v, 0.0f), 1.0f); }
__device__ inline float smooth(float lo, float hi, float x) {
    const float t = clamp01((x - lo) / (hi - lo));
    return t * t * (3.0f - 2.0f * t);
}

constexpr V3 kElectricTint{1.0f, 0.45f, 0.15f};
constexpr V3 kMagneticTint{0.20f, 0.65f, 1.0f};
constexpr V3 kGridTint{0.16f, 0.19f, 0.26f};
constexpr V3 kIntensityTint{1.0f, 0.8f, 0.45f};

__device__ inline uint64_t cell_of_coord(const ViewArgs &v, uint32_t x, uint32_t y, uint32_t z) {
    return (uint64_t(z) * v.n[1] + y) * v.pitch + x;
}

// sign(v) · log(1 + k|v|) / log(1 + k); linear when k <= 0.
__device__ inline float signed_log(float value, float strength) {
    if (strength <= 0.0f) return value;
    return signf(value) * logf(1.0f + strength * fabsf(value)) / logf(1.0f + strength);
}

// ½|E|² and ½|H|² at a cell.
__device__ inline void densities(const ViewArgs &v, uint64_t base, float &we, float &wh) {
    float se = 0.0f, sh = 0.0f;
    for (int c = 0; c < 3; ++c) {
        const float e = v.e[c * v.component_stride + base], h = v.h[c * v.component_stride + base];
        se += e * e;
        sh += h * h;
    }
    we = 0.5f * se;
    wh = 0.5f * sh;
}

__device__ inline float averaged_intensity(const ViewArgs &v, uint64_t base) {
    return v.intensity[base] / float(max(v.accumulated, 1u));
}

// World position in coarse cells to a fractional cell coordinate.
__device__ inline V3 cell_of(const ViewArgs &v, V3 point) {
    float out[3];
    for (int a = 0; a < 3; ++a) {
        const float fraction = clamp01(at(point, a) / v.box[a]);
        const float position = fraction * float(v.samples - 1u);
        const uint32_t low = uint32_t(position);
        const uint32_t high = min(low + 1u, v.samples - 1u);
        const float *section = v.lookup + size_t(a) * v.samples;
        out[a] = mixf(section[low], section[high], position - float(low));
    }
    return V3{out[0], out[1], out[2]};
}

__device__ inline V3 diverging(float value) {
    const V3 neutral{0.05f, 0.05f, 0.07f}, cold{0.25f, 0.48f, 1.0f}, hot{1.0f, 0.30f, 0.18f};
    const float magnitude = fminf(fabsf(value), 1.0f);
    return value < 0.0f ? mix3(neutral, cold, magnitude) : mix3(neutral, hot, magnitude);
}

__device__ inline V3 background(float sy) {
    const float shade = 0.5f + 0.5f * sy;
    return mix3(V3{0.02f, 0.02f, 0.03f}, V3{0.05f, 0.05f, 0.07f}, shade);
}

__device__ inline float edge_glow(V3 p, const float size[3]) {
    float d[3];
    for (int a = 0; a < 3; ++a) d[a] = fminf(at(p, a), size[a] - at(p, a)) / size[a];
    const float lo = fminf(fminf(d[0], d[1]), d[2]), hi = fmaxf(fmaxf(d[0], d[1]), d[2]);
    const float middle = d[0] + d[1] + d[2] - lo - hi;
    return smooth(0.01f, 0.0f, middle);
}

// The scrub bar along the bottom edge: colour and blend weight.
__device__ inline float scrub_bar(const ViewArgs &v, float sx, float sy, V3 &colour) {
    const float height = v.bar_height;
    if (height <= 0.0f) return 0.0f;
    const float from_bottom = 0.5f * (sy + 1.0f);
    if (from_bottom > height) return 0.0f;
    const float position = 0.5f * (sx + 1.0f);
    colour = V3{0.12f, 0.13f, 0.16f};
    if (position >= v.window_start) colour = V3{0.22f, 0.30f, 0.40f};
    if (position <= v.played) colour = V3{0.35f, 0.62f, 0.95f};
    if (fabsf(position - v.played) < 0.0025f) colour = V3{1.0f, 0.85f, 0.45f};
    const float softness = smooth(height, height * 0.6f, from_bottom);
    return 0.55f + 0.45f * softness;
}

__device__ inline V3 overlay(const ViewArgs &v, V3 field, float sx, float sy) {
    V3 bar{0.0f, 0.0f, 0.0f};
    const float alpha = scrub_bar(v, sx, sy, bar);
    return mix3(field, bar, alpha);
}

// Emission of the ribbon view at a fractional cell coordinate.
__device__ inline V3 ribbons(const ViewArgs &v, V3 cell) {
    const float extent[3] = {float(v.n[0]), float(v.n[1]), float(v.n[2])};
    const float middle[3] = {0.5f * extent[0], 0.5f * extent[1], 0.5f * extent[2]};
    const uint32_t ea = v.component_e, ha = v.component_h, travel = 3u - ea - ha;
    uint32_t probe[3] = {uint32_t(middle[0]), uint32_t(middle[1]), uint32_t(middle[2])};
    probe[travel] = min(uint32_t(fmaxf(at(cell, travel), 0.0f)), v.n[travel] - 1u);
    const uint64_t base = cell_of_coord(v, probe[0], probe[1], probe[2]);
    const float electric = v.e[ea * v.component_stride + base] * v.exposure;
    const float magnetic = v.h[ha * v.component_stride + base] * v.exposure;
    const float reach = 0.33f * extent[ea];
    const float thickness = 0.015f * extent[ea];
    const float from_e = at(cell, ea) - middle[ea];
    const float from_h = at(cell, ha) - middle[ha];
    V3 lit{0.0f, 0.0f, 0.0f};
    if (fabsf(from_h) < thickness && from_e * electric > 0.0f && fabsf(from_e) < fabsf(electric) * reach)
        lit = add(lit, kElectricTint);
    if (fabsf(from_e) < thickness && from_h * magnetic > 0.0f && fabsf(from_h) < fabsf(magnetic) * reach)
        lit = add(lit, kMagneticTint);
    if (fabsf(from_e) < thickness && fabsf(from_h) < thickness) lit = add(lit, V3{0.10f, 0.10f, 0.10f});
    return lit;
}

__device__ inline V3 emission(const ViewArgs &v, uint64_t base) {
    if (v.mode == kModeIntensity)
        return scale(kIntensityTint, signed_log(averaged_intensity(v, base) * v.exposure, v.log_strength));
    float we, wh;
    densities(v, base, we, wh);
    we *= v.exposure;
    wh *= v.exposure;
    if (v.mode == kModeMagnitude) {
        const float m = signed_log(we + wh, v.log_strength);
        return V3{m, m, m};
    }
    return add(scale(kElectricTint, signed_log(we, v.log_strength)), scale(kMagneticTint, signed_log(wh, v.log_strength)));
}

// IEC 61966-2-1 encoding of a linear value, as an sRGB render target stores it.
__device__ inline uint8_t srgb8(float linear) {
    const float c = clamp01(linear);
    const float s = c <= 0.0031308f ? 12.92f * c : 1.055f * powf(c, 1.0f / 2.4f) - 0.055f;
    return uint8_t(rintf(s * 255.0f));
}

__global__ void volume_pass(ViewArgs v) {
    const uint32_t px = blockIdx.x * blockDim.x + threadIdx.x, py = blockIdx.y * blockDim.y + threadIdx.y;
    if (px >= v.width || py >= v.height) return;
    // Pixel centre in normalized screen coordinates, +y up (row 0 is the top).
    const float sx = (float(px) + 0.5f) / float(v.width) * 2.0f - 1.0f;
    const float sy = 1.0f - (float(py) + 0.5f) / float(v.height) * 2.0f;
    V3 d{v.forward[0] + sx * v.right[0] + sy * v.up[0], v.forward[1] + sx * v.right[1] + sy * v.up[1],
         v.forward[2] + sx * v.right[2] + sy * v.up[2]};
    const float norm = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
    d = V3{d.x / norm, d.y / norm, d.z / norm};
    const V3 origin{v.origin[0], v.origin[1], v.origin[2]};
    const V3 sky = background(sy);

    // Slab-method intersection with the domain box.
    float near_t = -FLT_MAX, far_t = FLT_MAX;
    for (int a = 0; a < 3; ++a) {
        const float inverse = 1.0f / at(d, a);
        const float lo = (0.0f - at(origin, a)) * inverse, hi = (v.box[a] - at(origin, a)) * inverse;
        near_t = fmaxf(near_t, fminf(lo, hi));
        far_t = fminf(far_t, fmaxf(lo, hi));
    }
    const float enter = fmaxf(near_t, 0.0f);
    V3 colour;
    if (far_t <= enter) {
        colour = overlay(v, sky, sx, sy);
    } else {
        const float march = fmaxf(v.march, 0.25f);
        const bool signed_view = v.mode == kModeElectric || v.mode == kModeMagnetic || v.mode == kModeFields;
        V3 glow{0.0f, 0.0f, 0.0f};
        float extreme_x = 0.0f, extreme_y = 0.0f;
        float distance = enter + 0.5f * march;
        for (uint32_t taken = 0; taken < 4096u; ++taken) {
            if (distance >= far_t) break;
            const V3 point = add(origin, scale(d, distance));
            const V3 fractional = cell_of(v, point);
            uint32_t coord[3];
            for (int a = 0; a < 3; ++a) coord[a] = min(uint32_t(fmaxf(at(fractional, a), 0.0f)), v.n[a] - 1u);
            const uint64_t base = cell_of_coord(v, coord[0], coord[1], coord[2]);
            if (v.mode == kModeRibbons) {
                glow = add(glow, ribbons(v, fractional));
            } else if (v.mode == kModeGrid) {
                const float ex = fabsf(fractional.x - rintf(fractional.x));
                const float ey = fabsf(fractional.y - rintf(fractional.y));
                const float ez = fabsf(fractional.z - rintf(fractional.z));
                glow = add(glow, scale(kGridTint, smooth(0.08f, 0.0f, fminf(fminf(ex, ey), ez))));
            } else if (signed_view) {
                const float electric = v.e[v.component_e * v.component_stride + base];
                const float magnetic = v.h[v.component_h * v.component_stride + base];
                float vx, vy;
                if (v.mode == kModeFields) {
                    vx = electric * v.exposure;
                    vy = magnetic * v.exposure;
                } else {
                    vx = (v.mode == kModeMagnetic ? magnetic : electric) * v.exposure;
                    vy = 0.0f * v.exposure;
                }
                if (fabsf(vx) > fabsf(extreme_x)) extreme_x = vx;
                if (fabsf(vy) > fabsf(extreme_y)) extreme_y = vy;
            } else {
                glow = add(glow, emission(v, base));
            }
            distance += march;
        }
        const V3 rim = scale(V3{0.16f, 0.18f, 0.22f}, edge_glow(add(origin, scale(d, far_t)), v.box));
        V3 field;
        if (v.mode == kModeFields) {
            const float e = signed_log(extreme_x, v.log_strength), h = signed_log(extreme_y, v.log_strength);
            const V3 lit = add(scale(kElectricTint, fabsf(e)), scale(kMagneticTint, fabsf(h)));
            const V3 shade{0.5f + 0.5f * (signf(e) * fabsf(e)), 0.5f + 0.5f * 0.0f, 0.5f + 0.5f * (signf(h) * fabsf(h))};
            const float length = sqrtf(lit.x * lit.x + lit.y * lit.y + lit.z * lit.z);
            field = add(add(scale(sky, expf(-length)), mul(lit, shade)), rim);
        } else if (signed_view) {
            const float scaled = signed_log(extreme_x, v.log_strength);
            const float opacity = fminf(fabsf(scaled), 1.0f);
            field = add(add(scale(diverging(scaled), opacity), scale(sky, 1.0f - opacity)), rim);
        } else {
            glow = scale(glow, march * v.inverse_path);
            const V3 fade{expf(-glow.x), expf(-glow.y), expf(-glow.z)};
            const V3 opacity{1.0f - fade.x, 1.0f - fade.y, 1.0f - fade.z};
            field = add(add(opacity, mul(sky, fade)), rim);
        }
        colour = overlay(v, field, sx, sy);
    }
    uint8_t *out = v.image + (size_t(py) * v.width + px) * 4;
    out[0] = srgb8(colour.x);
    out[1] = srgb8(colour.y);
    out[2] = srgb8(colour.z);
    out[3] = 255;
}

// measure_peak: maxima over the real cells, by atomic max on the bit pattern
// (ordered like the value for non-negative floats).  Blocks walk whole rows,
// threads along them.  The averaged intensity's maximum is the maximum
// intensity divided once: dividing by a positive count is monotonic under
// round-to-nearest, so max(I / n) and max(I) / n are the same float.
__global__ void measure_peak(const float *e, const float *h, const float *intensity, uint64_t stride, uint32_t nx,
                             uint32_t ny, uint32_t nz, uint32_t pitch, uint32_t accumulated, uint32_t *peak) {
    float local[kPeakSlots] = {0, 0, 0, 0, 0, 0, 0, 0};
    float intensity_max = 0.0f;
    const uint64_t rows = uint64_t(ny) * nz;
    for (uint64_t row = blockIdx.x; row < rows; row += gridDim.x) {
        for (uint32_t x = threadIdx.x; x < nx; x += blockDim.x) {
            const uint64_t base = row * pitch + x;
            float se = 0.0f, sh = 0.0f;
            for (int c = 0; c < 3; ++c) {
                const float ev = e[c * stride + base], hv = h[c * stride + base];
                se += ev * ev;
                sh += hv * hv;
                local[1 + c] = fmaxf(local[1 + c], fabsf(ev));
                local[4 + c] = fmaxf(local[4 + c], fabsf(hv));
            }
            local[0] = fmaxf(local[0], fmaxf(0.5f * se, 0.5f * sh));
            intensity_max = fmaxf(intensity_max, intensity[base]);
        }
    }
    local[7] = intensity_max / float(max(accumulated, 1u));
    // Warp maxima, then block maxima in shared memory: one atomic per slot
    // per block (all blocks' atomics land on the same eight words).
    __shared__ float warp_max[kPeakSlots][32];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, warps = blockDim.x >> 5;
    for (int s = 0; s < kPeakSlots; ++s) {
        float m = local[s];
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) warp_max[s][warp] = m;
    }
    __syncthreads();
    if (threadIdx.x < kPeakSlots) {
        float m = 0.0f;
        for (int w = 0; w < warps; ++w) m = fmaxf(m, warp_max[threadIdx.x][w]);
        atomicMax(peak + threadIdx.x, __float_as_uint(m));
    }
}

} // namespace

struct dp_renderer {
    dp_sim *sim = nullptr;
    uint32_t width = 0, height = 0;
    uint8_t *image = nullptr;
    uint32_t *peak = nullptr;    // device, kPeakSlots
    uint32_t *peak_host = nullptr; // pinned copy of the last reduction
    float *lookup = nullptr;
    uint32_t samples = 0;
    float box[3] = {0, 0, 0};
    float scale = 0.0f;
    uint32_t components[2] = {2, 1};
    bool measured = false;

    ~dp_renderer() {
        if (sim && sim->stream) {
            cudaSetDevice(sim->device);
            cudaStreamSynchronize(sim->stream);
        }
        cudaFree(image);
        cudaFree(peak);
        cudaFree(lookup);
        cudaFreeHost(peak_host);
    }

    void measure() {
        const uint32_t *n = sim->scene.grid.n;
        check_cuda(cudaMemsetAsync(peak, 0, kPeakSlots * sizeof(uint32_t), sim->stream), "clear peak");
        const FieldSet f = sim->fields();
        const uint32_t accumulated = uint32_t(std::min<uint64_t>(sim->accumulated, 0xffffffffu));
        measure_peak<<<2048, 256, 0, sim->stream>>>(f.e, f.h, sim->intensity, sim->padded_cells(), n[0], n[1], n[2],
                                                    sim->pitch, accumulated, peak);
        check_cuda(cudaGetLastError(), "measure peak");
        check_cuda(cudaMemcpyAsync(peak_host, peak, kPeakSlots * sizeof(uint32_t), cudaMemcpyDeviceToHost, sim->stream),
                   "peak readback");
        measured = true;
    }

    // update_scale, render.rs:281-325: the previous reduction folded into a
    // running scale that rises quickly and falls slowly, and the dominant
    // component of each field.
    void update_scale(bool advanced, uint32_t mode) {
        if (!advanced || !measured) return;
        check_cuda(cudaStreamSynchronize(sim->stream), "peak wait");
        float slots[kPeakSlots];
        for (int s = 0; s < kPeakSlots; ++s) std::memcpy(&slots[s], &peak_host[s], 4);
        const float measured_peak = mode == kModeIntensity ? slots[7] : slots[0];
        auto dominant = [&](int offset) {
            int best = -1;
            for (int a = 0; a < 3; ++a) {
                const float v = slots[offset + a];
                if (!std::isfinite(v)) continue;
                if (best < 0 || !(v < slots[offset + best])) best = a; // the last of equal maxima
            }
            return uint32_t(best < 0 ? 0 : best);
        };
        const uint32_t electric = dominant(1);
        uint32_t magnetic = dominant(4);
        if (magnetic == electric) magnetic = (electric + 1) % 3;
        components[0] = electric;
        components[1] = magnetic;
        if (!std::isfinite(measured_peak) || measured_peak <= 0.0f) return;
        if (scale == 0.0f) {
            scale = measured_peak;
            return;
        }
        const float rate = measured_peak > scale ? 0.4f : 0.02f;
        scale += rate * (measured_peak - scale);
    }
};

namespace {

bool is_signed(uint32_t mode) {
    return mode == kModeElectric || mode == kModeMagnetic || mode == kModeRibbons || mode == kModeFields;
}

// Camera::basis (examples/common/camera.rs): an orbit around the box centre.
void camera_basis(const dp_view &view, const float box[3], float aspect, float position[3], float right[3],
                  float up[3], float forward[3]) {
    const float center[3] = {0.5f * box[0], 0.5f * box[1], 0.5f * box[2]};
    const float radius = std::max(std::max(box[0], box[1]), box[2]);
    const float sp = std::sin(view.pitch), cp = std::cos(view.pitch);
    const float sy = std::sin(view.yaw), cy = std::cos(view.yaw);
    const float away[3] = {cp * sy, sp, cp * cy};
    for (int a = 0; a < 3; ++a) {
        position[a] = center[a] + away[a] * view.distance * radius;
        forward[a] = -away[a];
    }
    const float world_up[3] = {0.0f, 1.0f, 0.0f};
    float r[3] = {forward[1] * world_up[2] - forward[2] * world_up[1], forward[2] * world_up[0] - forward[0] * world_up[2],
                  forward[0] * world_up[1] - forward[1] * world_up[0]};
    const float norm = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    for (float &c : r) c = c / norm;
    const float u[3] = {r[1] * forward[2] - r[2] * forward[1], r[2] * forward[0] - r[0] * forward[2],
                        r[0] * forward[1] - r[1] * forward[0]};
    const float tangent = std::tan(0.5f * view.fov);
    for (int a = 0; a < 3; ++a) {
        right[a] = r[a] * tangent * aspect;
        up[a] = u[a] * tangent;
    }
}

} // namespace

extern "C" {

dp_view dp_view_default(void) {
    dp_view v{};
    v.yaw = 0.9f;
    v.pitch = 0.45f;
    v.distance = 1.9f;
    v.fov = 0.8f;
    v.mode = DP_VIEW_FIELDS;
    v.gain = 1.0f;
    v.log_strength = 6.0f;
    v.scrub = 0;
    return v;
}

dp_status dp_renderer_create(dp_sim *sim, uint32_t width, uint32_t height, dp_renderer **out) {
    return guarded([&] {
        if (!sim || !out) throw Error(DP_ERR_INVALID, "null argument");
        *out = nullptr;
        if (width == 0 || height == 0 || width > 16384 || height > 16384) throw Error(DP_ERR_RANGE, "image size out of range");
        auto r = std::make_unique<dp_renderer>();
        r->sim = sim;
        r->width = width;
        r->height = height;
        sim->bind();
        const Scene &s = sim->scene;
        // The world-to-cell table at the reference GPU solver's sample count.
        r->samples = s.lookup_samples();
        const std::vector<float> lookup = s.cell_lookup(r->samples);
        for (int a = 0; a < 3; ++a) r->box[a] = s.grid.axes[a].length() / s.grid.base; // Grid::box_size
        check_cuda(cudaMalloc(&r->lookup, lookup.size() * sizeof(float)), "lookup");
        check_cuda(cudaMemcpy(r->lookup, lookup.data(), lookup.size() * sizeof(float), cudaMemcpyHostToDevice), "lookup");
        check_cuda(cudaMalloc(&r->image, size_t(width) * height * 4), "image");
        check_cuda(cudaMalloc(&r->peak, kPeakSlots * sizeof(uint32_t)), "peak");
        check_cuda(cudaMallocHost(&r->peak_host, kPeakSlots * sizeof(uint32_t)), "peak");
        *out = r.release();
        return DP_OK;
    });
}

void dp_renderer_destroy(dp_renderer *r) { delete r; }

dp_status dp_renderer_measure(dp_renderer *r) {
    return guarded([&] {
        if (!r) throw Error(DP_ERR_INVALID, "null handle");
        r->sim->bind();
        r->measure();
        return DP_OK;
    });
}

dp_status dp_renderer_draw(dp_renderer *r, const dp_view *view, int32_t advanced) {
    return guarded([&] {
        if (!r || !view) throw Error(DP_ERR_INVALID, "null argument");
        if (view->mode > DP_VIEW_INTENSITY) throw Error(DP_ERR_INVALID, "unknown view mode");
        dp_sim *sim = r->sim;
        sim->bind();
        r->update_scale(advanced != 0, view->mode);
        r->measure();
        ViewArgs v{};
        const FieldSet f = sim->fields();
        v.e = f.e;
        v.h = f.h;
        v.intensity = sim->intensity;
        v.component_stride = sim->padded_cells();
        for (int a = 0; a < 3; ++a) {
            v.n[a] = sim->scene.grid.n[a];
            v.box[a] = r->box[a];
        }
        v.pitch = sim->pitch;
        v.lookup = r->lookup;
        v.samples = r->samples;
        const float aspect = float(r->width) / float(std::max(r->height, 1u));
        camera_basis(*view, r->box, aspect, v.origin, v.right, v.up, v.forward);
        v.march = 1.0f; // one sample per cell (render.rs:426-428)
        const float reference = std::max(r->scale, FLT_MIN);
        v.exposure = is_signed(view->mode) ? view->gain / std::sqrt(2.0f * reference) : view->gain / reference;
        v.log_strength = view->log_strength;
        v.mode = view->mode;
        const float longest = std::max(std::max(r->box[0], r->box[1]), r->box[2]);
        v.inverse_path = 1.0f / std::max(longest / 3.0f, 1.0f); // reference_path, render.rs:480-488
        if (view->scrub) {
            v.played = view->played;
            v.window_start = view->window_start;
            v.bar_height = 0.045f;
        }
        v.component_e = r->components[0];
        v.component_h = r->components[1];
        v.accumulated = uint32_t(std::min<uint64_t>(sim->accumulated, 0xffffffffu));
        v.width = r->width;
        v.height = r->height;
        v.image = r->image;
        const dim3 block(16, 16), grid((r->width + 15) / 16, (r->height + 15) / 16);
        volume_pass<<<grid, block, 0, sim->stream>>>(v);
        check_cuda(cudaGetLastError(), "volume pass");
        return DP_OK;
    });
}

dp_status dp_renderer_pixels(dp_renderer *r, uint8_t *host, size_t bytes) {
    return guarded([&] {
        if (!r || !host) throw Error(DP_ERR_INVALID, "null argument");
        if (bytes != size_t(r->width) * r->height * 4) throw Error(DP_ERR_RANGE, "buffer size does not match the image");
        r->sim->bind();
        check_cuda(cudaMemcpyAsync(host, r->image, bytes, cudaMemcpyDeviceToHost, r->sim->stream), "pixels");
        check_cuda(cudaStreamSynchronize(r->sim->stream), "pixels");
        return DP_OK;
    });
}

dp_status dp_renderer_image(dp_renderer *r, void **device_rgba) {
    return guarded([&] {
        if (!r || !device_rgba) throw Error(DP_ERR_INVALID, "null argument");
        *device_rgba = r->image;
        return DP_OK;
    });
}

dp_status dp_renderer_state(dp_renderer *r, float peaks[8], float *scale, uint32_t components[2]) {
    return guarded([&] {
        if (!r) throw Error(DP_ERR_INVALID, "null handle");
        r->sim->bind();
        check_cuda(cudaStreamSynchronize(r->sim->stream), "peak wait");
        if (peaks)
            for (int s = 0; s < kPeakSlots; ++s) std::memcpy(&peaks[s], &r->peak_host[s], 4);
        if (scale) *scale = r->scale;
        if (components) {
            components[0] = r->components[0];
            components[1] = r->components[1];
        }
        return DP_OK;
    });
}

} // extern "C"
