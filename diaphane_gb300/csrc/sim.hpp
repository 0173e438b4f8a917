// The simulation handle (gpu::Simulation, src/gpu.rs:159-763), shared by the
// C ABI translation units that operate on it (sim.cu, keyframes.cu).
//
// A handle owns its device tables, two field buffer sets and one stream.
// The fused step reads one set and writes the other (ping-pong), which is
// what lets H and E of a whole step be computed in a single pass over HBM.
// The naive passes and the reverse step work in place on the current set.
#pragma once

#include "abi.hpp"
#include "device.cuh"
#include "profiles.hpp"

#include <algorithm>
#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

namespace diaphane {
const Scene &scene_of(const dp_scene *s);

inline void check_cuda(cudaError_t err, const char *what) {
    if (err != cudaSuccess) {
        cudaGetLastError();
        throw Error(err == cudaErrorMemoryAllocation ? DP_ERR_OOM : DP_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(err));
    }
}

// Probe gather (sim.cu): Ez and Hy at `count` padded cell indices into slot
// `slot` of a ring of per-step records.
void launch_probe_gather(const float *e, const float *h, uint64_t cells, const uint32_t *probe_cells, uint32_t count,
                         float *ring, uint64_t slot, cudaStream_t stream);
} // namespace diaphane

using namespace diaphane;

struct dp_sim {
    Scene scene;
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t kernel = DP_KERNEL_NAIVE;
    DeviceScene dev{};
    FieldSet set[2]{};
    int current = 0;
    float *intensity = nullptr;
    float *primary = nullptr;
    float *dual = nullptr;
    float2 *eps_mu = nullptr;
    double *partials = nullptr;
    double *host_partials = nullptr;
    int32_t *flag = nullptr;
    int32_t *error = nullptr;        // set by a kernel whose bounded wait gave up
    uint8_t *material_padded = nullptr;
    uint32_t material_pitch = 0;
    uint32_t pitch = 0;              // field row stride in cells (nx rounded up to 4)
    FusedPlan plan{};
    FusedMaps maps[2]{};             // tensor maps reading set 0 / set 1
    std::vector<void *> owned;
    uint64_t step = 0;
    uint64_t accumulated = 0;
    bool accumulating = false;
    uint64_t launches = 0;
    std::vector<StepInjection> injections;
    // Total-field boxes: their incident lines and the per-step profile values
    // of the side faces, staged to the device (null when the step has none).
    IncidentLines<float> lines;
    ProfileRing<float> profile_ring;
    std::vector<float> profile_values;
    const float *step_profiles = nullptr;
    // Probes: Ez and Hy at given cells after every step, in a device ring of
    // probe_capacity steps.  Records are valid for steps after probe_since
    // (a restore, reverse or reset starts a new history).
    uint32_t *probe_cells = nullptr; // padded linear cell indices
    uint32_t probe_count = 0;
    uint64_t probe_capacity = 0;
    float *probe_ring = nullptr;     // capacity × count × (Ez, Hy)
    uint64_t probe_since = 0;

    ~dp_sim() {
        if (stream) {
            cudaSetDevice(device);
            cudaStreamSynchronize(stream);
        }
        cudaFree(probe_cells);
        cudaFree(probe_ring);
        for (void *p : owned) cudaFree(p);
        if (host_partials) cudaFreeHost(host_partials);
        if (stream) cudaStreamDestroy(stream);
    }

    void bind() { diaphane::check_cuda(cudaSetDevice(device), "cudaSetDevice"); }

    FieldSet fields() const { return set[current]; }

    // The non-silent injections of step `at_step` (at `time`), in
    // application order (apply_sources, src/cpu.rs:606-633).
    void collect(uint64_t at_step, float time, std::vector<DeviceInjection> &out) {
        out.clear();
        const std::vector<BoxCorrections<float>> *boxes = lines.empty() ? nullptr : &lines.at(at_step);
        scene.injections_in<float>(time, injections, boxes, &profile_values);
        step_profiles = profile_values.empty() ? nullptr : profile_ring.put(profile_values, stream);
        for (const StepInjection &s : injections) {
            if (s.value == 0.0f) continue;
            DeviceInjection d{};
            for (int a = 0; a < 3; ++a) {
                d.origin[a] = s.origin[a];
                d.extent[a] = s.extent[a];
            }
            d.component = s.component;
            d.magnetic = s.magnetic;
            d.value = s.value;
            d.weight_offset = s.weight_offset;
            d.profile_offset = s.profile_offset;
            d.profile_axis = s.profile_axis;
            out.push_back(d);
        }
    }

    void inject_phase(const std::vector<DeviceInjection> &all, bool magnetic, float sign) {
        for (const DeviceInjection &d : all) {
            if (bool(d.magnetic) != magnetic) continue;
            launch_inject(dev, fields(), d, sign, step_profiles, stream);
            ++launches;
        }
    }

    // advance (src/cpu.rs:174-198, src/gpu.rs:425-481).
    void forward(uint64_t steps) {
        std::vector<DeviceInjection> all;
        for (uint64_t n = 0; n < steps; ++n) {
            // `E` holds (step + 1)·dt after its update; injections are stated
            // relative to that instant.
            const float time = float(step + 1) * scene.dt;
            collect(step, time, all);
            if (kernel == DP_KERNEL_FUSED) {
                InjectionTable table{};
                table.count = uint32_t(all.size());
                table.profiles = step_profiles;
                for (size_t k = 0; k < all.size(); ++k) table.item[k] = all[k];
                launch_fused_step(dev, plan, maps[current], set[current ^ 1], accumulating ? intensity : nullptr,
                                  table, error, stream);
                ++launches;
                current ^= 1;
            } else {
                launch_naive_magnetic(dev, fields(), false, stream);
                ++launches;
                inject_phase(all, true, 1.0f);
                launch_naive_electric(dev, fields(), false, stream);
                ++launches;
                inject_phase(all, false, 1.0f);
                if (accumulating) {
                    launch_intensity(dev, fields().e, intensity, stream);
                    ++launches;
                }
            }
            diaphane::check_cuda(cudaGetLastError(), "step launch");
            if (accumulating) ++accumulated;
            ++step;
            if (probe_count) {
                launch_probe_gather(fields().e, fields().h, padded_cells(), probe_cells, probe_count, probe_ring,
                                    (step - 1) % probe_capacity, stream);
                ++launches;
            }
        }
    }

    // reverse (src/cpu.rs:253-273, src/gpu.rs:537-573): each forward phase
    // undone in the opposite order with the drive negated.
    void backward(uint64_t steps) {
        std::vector<DeviceInjection> all;
        for (uint64_t n = 0; n < steps; ++n) {
            const float time = float(step) * scene.dt;
            collect(step - 1, time, all);
            inject_phase(all, false, -1.0f);
            launch_naive_electric(dev, fields(), true, stream);
            ++launches;
            inject_phase(all, true, -1.0f);
            launch_naive_magnetic(dev, fields(), true, stream);
            ++launches;
            diaphane::check_cuda(cudaGetLastError(), "reverse launch");
            --step;
            probe_since = std::min(probe_since, step);
        }
    }

    uint64_t padded_cells() const { return uint64_t(pitch) * scene.grid.n[1] * scene.grid.n[2]; }

    // Back to step 0 with empty fields (reset, src/gpu.rs:586-603).
    void reset_fields() {
        const uint64_t cells = padded_cells();
        for (int k = 0; k < 2; ++k) {
            diaphane::check_cuda(cudaMemsetAsync(set[k].e, 0, 3 * cells * sizeof(float), stream), "reset");
            diaphane::check_cuda(cudaMemsetAsync(set[k].h, 0, 3 * cells * sizeof(float), stream), "reset");
        }
        diaphane::check_cuda(cudaMemsetAsync(intensity, 0, cells * sizeof(float), stream), "reset");
        current = 0;
        step = 0;
        accumulated = 0;
        probe_since = 0;
    }

    void clear_intensity() {
        if (accumulated == 0) return;
        diaphane::check_cuda(cudaMemsetAsync(intensity, 0, padded_cells() * sizeof(float), stream), "clear intensity");
        accumulated = 0;
    }

    // Dense host rows <-> pitched device rows, `components` of them.
    void copy_out(float *host, const float *device, int components) {
        try {
            copy_fields_out(host, device, scene.grid.n, pitch, padded_cells(), components, stream);
        } catch (const std::runtime_error &e) {
            throw Error(DP_ERR_CUDA, e.what());
        }
    }
    void copy_in(float *device, const float *host, int components) {
        try {
            copy_fields_in(device, host, scene.grid.n, pitch, padded_cells(), components, stream);
        } catch (const std::runtime_error &e) {
            throw Error(DP_ERR_CUDA, e.what());
        }
    }

    void wait(uint32_t timeout_ms) {
        const cudaError_t q = poll_stream(stream, timeout_ms);
        if (q == cudaErrorNotReady) throw Error(DP_ERR_TIMEOUT, "the GPU did not finish in time");
        diaphane::check_cuda(q, "stream");
        if (kernel == DP_KERNEL_FUSED) {
            int32_t code = 0;
            diaphane::check_cuda(cudaMemcpy(&code, error, sizeof(code), cudaMemcpyDeviceToHost), "error flag");
            if (code != 0) {
                diaphane::check_cuda(cudaMemset(error, 0, sizeof(int32_t)), "error flag");
                throw Error(DP_ERR_TIMEOUT, "a fused step gave up waiting for its plane loads");
            }
        }
    }
};

