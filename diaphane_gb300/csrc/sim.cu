// C ABI: the simulation handle (gpu::Simulation, src/gpu.rs:159-763).
//
// A handle owns its device tables, two field buffer sets and one stream.
// The fused step reads one set and writes the other (ping-pong), which is
// what lets H and E of a whole step be computed in a single pass over HBM.
// The naive passes and the reverse step work in place on the current set.
#include "abi.hpp"
#include "device.cuh"

#include <chrono>
#include <cstring>
#include <thread>
#include <vector>

namespace diaphane {
const Scene &scene_of(const dp_scene *s);
}

using namespace diaphane;

namespace {

void check(cudaError_t err, const char *what) {
    if (err != cudaSuccess) {
        cudaGetLastError();
        throw Error(err == cudaErrorMemoryAllocation ? DP_ERR_OOM : DP_ERR_CUDA,
                    std::string(what) + ": " + cudaGetErrorString(err));
    }
}

template <typename T> T *device_alloc(size_t count, std::vector<void *> &owned) {
    void *p = nullptr;
    if (count == 0) count = 1;
    check(cudaMalloc(&p, count * sizeof(T)), "cudaMalloc");
    owned.push_back(p);
    return static_cast<T *>(p);
}

template <typename T> T *device_upload(const std::vector<T> &host, std::vector<void *> &owned, cudaStream_t stream) {
    T *p = device_alloc<T>(host.size(), owned);
    if (!host.empty())
        check(cudaMemcpyAsync(p, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice, stream), "upload");
    return p;
}

} // namespace

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

    ~dp_sim() {
        if (stream) {
            cudaSetDevice(device);
            cudaStreamSynchronize(stream);
        }
        for (void *p : owned) cudaFree(p);
        if (host_partials) cudaFreeHost(host_partials);
        if (stream) cudaStreamDestroy(stream);
    }

    void bind() { check(cudaSetDevice(device), "cudaSetDevice"); }

    FieldSet fields() const { return set[current]; }

    // The non-silent injections of one phase at `time`, in application order
    // (apply_sources, src/cpu.rs:606-633).
    void collect(float time, std::vector<DeviceInjection> &out) {
        out.clear();
        scene.injections(time, injections);
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
            out.push_back(d);
        }
    }

    void inject_phase(const std::vector<DeviceInjection> &all, bool magnetic, float sign) {
        for (const DeviceInjection &d : all) {
            if (bool(d.magnetic) != magnetic) continue;
            launch_inject(dev, fields(), d, sign, stream);
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
            collect(time, all);
            if (kernel == DP_KERNEL_FUSED) {
                InjectionTable table{};
                table.count = uint32_t(all.size());
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
            check(cudaGetLastError(), "step launch");
            if (accumulating) ++accumulated;
            ++step;
        }
    }

    // reverse (src/cpu.rs:253-273, src/gpu.rs:537-573): each forward phase
    // undone in the opposite order with the drive negated.
    void backward(uint64_t steps) {
        std::vector<DeviceInjection> all;
        for (uint64_t n = 0; n < steps; ++n) {
            const float time = float(step) * scene.dt;
            collect(time, all);
            inject_phase(all, false, -1.0f);
            launch_naive_electric(dev, fields(), true, stream);
            ++launches;
            inject_phase(all, true, -1.0f);
            launch_naive_magnetic(dev, fields(), true, stream);
            ++launches;
            check(cudaGetLastError(), "reverse launch");
            --step;
        }
    }

    uint64_t padded_cells() const { return uint64_t(pitch) * scene.grid.n[1] * scene.grid.n[2]; }

    void clear_intensity() {
        if (accumulated == 0) return;
        check(cudaMemsetAsync(intensity, 0, padded_cells() * sizeof(float), stream), "clear intensity");
        accumulated = 0;
    }

    // Dense host rows <-> pitched device rows, `components` of them.
    void copy_out(float *host, const float *device, int components) {
        const uint32_t *n = scene.grid.n;
        const uint64_t dense = scene.grid.cells(), padded = padded_cells();
        for (int c = 0; c < components; ++c)
            check(cudaMemcpy2DAsync(host + c * dense, size_t(n[0]) * 4, device + c * padded, size_t(pitch) * 4,
                                    size_t(n[0]) * 4, size_t(n[1]) * n[2], cudaMemcpyDeviceToHost, stream),
                  "readback");
    }
    void copy_in(float *device, const float *host, int components) {
        const uint32_t *n = scene.grid.n;
        const uint64_t dense = scene.grid.cells(), padded = padded_cells();
        for (int c = 0; c < components; ++c)
            check(cudaMemcpy2DAsync(device + c * padded, size_t(pitch) * 4, host + c * dense, size_t(n[0]) * 4,
                                    size_t(n[0]) * 4, size_t(n[1]) * n[2], cudaMemcpyHostToDevice, stream),
                  "upload");
    }

    void wait(uint32_t timeout_ms) {
        const auto deadline = std::chrono::steady_clock::now() + std::chrono::milliseconds(timeout_ms);
        for (;;) {
            cudaError_t q = cudaStreamQuery(stream);
            if (q == cudaSuccess) break;
            if (q != cudaErrorNotReady) check(q, "stream");
            if (std::chrono::steady_clock::now() >= deadline) throw Error(DP_ERR_TIMEOUT, "the GPU did not finish in time");
            std::this_thread::sleep_for(std::chrono::microseconds(50));
        }
        if (kernel == DP_KERNEL_FUSED) {
            int32_t code = 0;
            check(cudaMemcpy(&code, error, sizeof(code), cudaMemcpyDeviceToHost), "error flag");
            if (code != 0) {
                check(cudaMemset(error, 0, sizeof(int32_t)), "error flag");
                throw Error(DP_ERR_TIMEOUT, "a fused step gave up waiting for its plane loads");
            }
        }
    }
};

namespace {

constexpr uint32_t kDefaultTimeoutMs = 120000; // src/gpu.rs:184

dp_sim *make_sim(const Scene &scene, const dp_options *opts) {
    auto sim = std::make_unique<dp_sim>();
    sim->scene = scene;
    sim->device = opts ? opts->device : 0;
    int count = 0;
    check(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
    if (sim->device < 0 || sim->device >= count) throw Error(DP_ERR_CUDA, "no such CUDA device");
    sim->bind();
    check(cudaStreamCreateWithFlags(&sim->stream, cudaStreamNonBlocking), "cudaStreamCreate");

    const Scene &s = sim->scene;
    // Rows are padded to a multiple of 4 cells (16 bytes) so the fused step's
    // tensor maps can stride them; for such grids the layout is the
    // reference's dense one exactly.
    const uint32_t nx = s.grid.n[0];
    sim->pitch = (nx + 3) / 4 * 4;
    const uint64_t cells = uint64_t(sim->pitch) * s.grid.n[1] * s.grid.n[2];
    auto &owned = sim->owned;
    cudaStream_t st = sim->stream;

    uint32_t requested = opts ? opts->kernel : DP_KERNEL_AUTO;
    if (requested > DP_KERNEL_NAIVE) throw Error(DP_ERR_INVALID, "unknown kernel selector");
    const bool fits = tensor_maps_available() && 2 * s.sources.size() <= size_t(kMaxInjections);
    if (requested == DP_KERNEL_FUSED && !fits)
        throw Error(DP_ERR_UNSUPPORTED, "the fused step does not cover this grid shape or source count");
    sim->kernel = (requested == DP_KERNEL_NAIVE || !fits) ? DP_KERNEL_NAIVE : DP_KERNEL_FUSED;

    DeviceScene &d = sim->dev;
    for (int a = 0; a < 3; ++a) d.n[a] = s.grid.n[a];
    d.pitch = sim->pitch;
    d.cells = cells;
    {
        // The index is rasterized on the device, straight into its buffer.
        uint8_t *material = device_alloc<uint8_t>(cells, owned);
        rasterize_on_device(s, material, sim->pitch, st);
        d.material = material;
    }
    // Padded to all 256 u8 indices, so a kernel may stage the whole table.
    std::vector<float4> coeff(256, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
    for (size_t m = 0; m < s.coefficients.size(); ++m) {
        const Coeff &c = s.coefficients[m];
        coeff[m] = make_float4(c.electric_gain, c.electric_loss, c.magnetic_gain, c.magnetic_loss);
    }
    d.coeff = device_upload(coeff, owned, st);
    d.mgain = device_upload(s.magnetic_gains, owned, st);
    d.egain = device_upload(s.electric_gains, owned, st);
    d.absorber = device_upload(s.absorber, owned, st);
    d.weights = device_upload(s.weights, owned, st);
    sim->primary = device_upload(s.primary, owned, st);
    sim->dual = device_upload(s.dual, owned, st);
    std::vector<float2> eps_mu;
    for (const dp_material &m : s.materials) eps_mu.push_back(make_float2(m.relative_permittivity, m.relative_permeability));
    sim->eps_mu = device_upload(eps_mu, owned, st);

    const int sets = sim->kernel == DP_KERNEL_FUSED ? 2 : 1;
    for (int k = 0; k < sets; ++k) {
        sim->set[k].e = device_alloc<float>(3 * cells, owned);
        sim->set[k].h = device_alloc<float>(3 * cells, owned);
        check(cudaMemsetAsync(sim->set[k].e, 0, 3 * cells * sizeof(float), st), "memset");
        check(cudaMemsetAsync(sim->set[k].h, 0, 3 * cells * sizeof(float), st), "memset");
    }
    if (sets == 1) sim->set[1] = sim->set[0];
    sim->intensity = device_alloc<float>(cells, owned);
    check(cudaMemsetAsync(sim->intensity, 0, cells * sizeof(float), st), "memset");
    const uint32_t blocks = energy_blocks(cells);  // padded cells
    sim->partials = device_alloc<double>(2 * size_t(blocks), owned);
    check(cudaMallocHost(&sim->host_partials, 2 * size_t(blocks) * sizeof(double)), "cudaMallocHost");
    sim->flag = device_alloc<int32_t>(1, owned);
    sim->error = device_alloc<int32_t>(1, owned);
    check(cudaMemsetAsync(sim->error, 0, sizeof(int32_t), st), "memset");

    if (sim->kernel == DP_KERNEL_FUSED) {
        int sms = 0;
        check(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sim->device), "attribute");
        try {
            sim->plan = fused_plan(s.grid.n, opts ? opts->cells_per_lane : 0, opts ? opts->tile_y : 0,
                                   opts ? opts->ring_slots : 0, opts ? opts->z_chunk : 0, sms);
        } catch (const std::exception &e) {
            throw Error(DP_ERR_UNSUPPORTED, e.what());
        }
        // The index again with rows padded to 16 bytes, for its tensor map.
        const uint64_t rows = uint64_t(s.grid.n[1]) * s.grid.n[2];
        sim->material_pitch = (nx + 15) / 16 * 16;
        sim->material_padded = device_alloc<uint8_t>(size_t(sim->material_pitch) * rows, owned);
        rasterize_on_device(s, sim->material_padded, sim->material_pitch, st);
        check(cudaStreamSynchronize(st), "setup upload");
        try {
            for (int k = 0; k < 2; ++k)
                fused_maps(d, sim->plan, sim->set[k], sim->material_padded, sim->material_pitch, sim->maps[k]);
        } catch (const std::exception &e) {
            throw Error(DP_ERR_CUDA, e.what());
        }
    }
    check(cudaStreamSynchronize(st), "setup upload");
    return sim.release();
}

size_t field_count(const dp_sim *sim, uint32_t field) {
    const uint64_t cells = sim->scene.grid.cells();
    return field == DP_FIELD_INTENSITY ? cells : 3 * cells;
}

float *field_ptr(dp_sim *sim, uint32_t field) {
    switch (field) {
    case DP_FIELD_ELECTRIC: return sim->fields().e;
    case DP_FIELD_MAGNETIC: return sim->fields().h;
    case DP_FIELD_INTENSITY: return sim->intensity;
    }
    throw Error(DP_ERR_INVALID, "unknown field");
}

} // namespace

extern "C" {

dp_status dp_sim_create(const dp_scene *scene, const dp_options *opts, dp_sim **out) {
    return guarded([&] {
        if (!scene || !out) throw Error(DP_ERR_INVALID, "null argument");
        *out = nullptr;
        *out = make_sim(scene_of(scene), opts);
        return DP_OK;
    });
}

void dp_sim_destroy(dp_sim *sim) { delete sim; }

dp_status dp_sim_advance(dp_sim *sim, uint64_t steps) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        sim->bind();
        sim->forward(steps);
        return DP_OK;
    });
}

dp_status dp_sim_reverse(dp_sim *sim, uint64_t steps) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        if (steps == 0) return DP_OK;
        if (!sim->scene.reversible)
            throw Error(DP_ERR_LOSSY, "this scene is lossy, and running a dissipative update backwards amplifies "
                                      "roundoff exponentially; reversal needs Boundary::Pec and no conductive material");
        if (sim->step < steps) throw Error(DP_ERR_RANGE, "cannot step back past the start");
        sim->bind();
        sim->clear_intensity();
        sim->backward(steps);
        return DP_OK;
    });
}

dp_status dp_sim_reset(dp_sim *sim) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        sim->bind();
        const uint64_t cells = sim->padded_cells();
        for (int k = 0; k < 2; ++k) {
            check(cudaMemsetAsync(sim->set[k].e, 0, 3 * cells * sizeof(float), sim->stream), "reset");
            check(cudaMemsetAsync(sim->set[k].h, 0, 3 * cells * sizeof(float), sim->stream), "reset");
        }
        check(cudaMemsetAsync(sim->intensity, 0, cells * sizeof(float), sim->stream), "reset");
        sim->current = 0;
        sim->step = 0;
        sim->accumulated = 0;
        return DP_OK;
    });
}

dp_status dp_sim_wait(dp_sim *sim, uint32_t timeout_ms) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        sim->bind();
        sim->wait(timeout_ms);
        return DP_OK;
    });
}

uint64_t dp_sim_step_count(const dp_sim *sim) { return sim ? sim->step : 0; }

float dp_sim_time(const dp_sim *sim) { return sim ? float(sim->step) * sim->scene.dt : 0.0f; }

dp_status dp_sim_read_field(dp_sim *sim, uint32_t field, float *host, size_t count) {
    return guarded([&] {
        if (!sim || !host) throw Error(DP_ERR_INVALID, "null argument");
        if (count != field_count(sim, field)) throw Error(DP_ERR_RANGE, "element count does not match the field");
        sim->bind();
        sim->wait(kDefaultTimeoutMs);
        sim->copy_out(host, field_ptr(sim, field), field == DP_FIELD_INTENSITY ? 1 : 3);
        sim->wait(kDefaultTimeoutMs);
        return DP_OK;
    });
}

dp_status dp_sim_write_field(dp_sim *sim, uint32_t field, const float *host, size_t count) {
    return guarded([&] {
        if (!sim || !host) throw Error(DP_ERR_INVALID, "null argument");
        if (count != field_count(sim, field)) throw Error(DP_ERR_RANGE, "snapshot was taken from a different grid");
        sim->bind();
        sim->wait(kDefaultTimeoutMs);
        sim->copy_in(field_ptr(sim, field), host, field == DP_FIELD_INTENSITY ? 1 : 3);
        sim->wait(kDefaultTimeoutMs);
        return DP_OK;
    });
}

dp_status dp_sim_restore(dp_sim *sim, uint64_t step, const float *electric, const float *magnetic, size_t count) {
    return guarded([&] {
        if (!sim || !electric || !magnetic) throw Error(DP_ERR_INVALID, "null argument");
        if (count != 3 * sim->scene.grid.cells()) throw Error(DP_ERR_RANGE, "snapshot was taken from a different grid");
        sim->bind();
        // The average belongs to the history that was just abandoned.
        sim->clear_intensity();
        sim->wait(kDefaultTimeoutMs);
        sim->copy_in(sim->fields().e, electric, 3);
        sim->copy_in(sim->fields().h, magnetic, 3);
        sim->wait(kDefaultTimeoutMs);
        sim->step = step;
        return DP_OK;
    });
}

dp_status dp_sim_set_accumulate_intensity(dp_sim *sim, int on) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        sim->bind();
        if (on && !sim->accumulating) sim->clear_intensity();
        sim->accumulating = on != 0;
        return DP_OK;
    });
}

uint64_t dp_sim_accumulated_steps(const dp_sim *sim) { return sim ? sim->accumulated : 0; }

dp_status dp_sim_device_ptr(dp_sim *sim, uint32_t field, void **ptr) {
    return guarded([&] {
        if (!sim || !ptr) throw Error(DP_ERR_INVALID, "null argument");
        *ptr = field_ptr(sim, field);
        return DP_OK;
    });
}

dp_status dp_sim_stream(dp_sim *sim, void **stream) {
    return guarded([&] {
        if (!sim || !stream) throw Error(DP_ERR_INVALID, "null argument");
        *stream = sim->stream;
        return DP_OK;
    });
}

uint64_t dp_sim_bytes_per_step(const dp_sim *sim) { return sim ? 48 * sim->scene.grid.cells() : 0; }

uint64_t dp_sim_field_bytes(const dp_sim *sim) { return sim ? 12 * sim->scene.grid.cells() : 0; }

dp_status dp_sim_energy(dp_sim *sim, double *electric, double *magnetic) {
    return guarded([&] {
        if (!sim || !electric || !magnetic) throw Error(DP_ERR_INVALID, "null argument");
        sim->bind();
        const uint32_t blocks = energy_blocks(sim->padded_cells());
        launch_energy(sim->dev, sim->fields(), sim->primary, sim->dual, sim->eps_mu, sim->partials, blocks, sim->stream);
        ++sim->launches;
        check(cudaGetLastError(), "energy launch");
        check(cudaMemcpyAsync(sim->host_partials, sim->partials, 2 * size_t(blocks) * sizeof(double),
                              cudaMemcpyDeviceToHost, sim->stream),
              "energy readback");
        sim->wait(kDefaultTimeoutMs);
        double e = 0.0, m = 0.0;
        for (uint32_t b = 0; b < blocks; ++b) {
            e += sim->host_partials[2 * b];
            m += sim->host_partials[2 * b + 1];
        }
        *electric = e;
        *magnetic = m;
        return DP_OK;
    });
}

dp_status dp_sim_is_finite(dp_sim *sim, int32_t *finite) {
    return guarded([&] {
        if (!sim || !finite) throw Error(DP_ERR_INVALID, "null argument");
        sim->bind();
        const int32_t one = 1;
        check(cudaMemcpyAsync(sim->flag, &one, sizeof(one), cudaMemcpyHostToDevice, sim->stream), "flag");
        launch_finite(sim->dev, sim->fields(), sim->flag, sim->stream);
        ++sim->launches;
        check(cudaGetLastError(), "finite launch");
        int32_t value = 0;
        check(cudaMemcpyAsync(&value, sim->flag, sizeof(value), cudaMemcpyDeviceToHost, sim->stream), "flag");
        sim->wait(kDefaultTimeoutMs);
        *finite = value;
        return DP_OK;
    });
}

int32_t dp_sim_is_reversible(const dp_sim *sim) { return sim && sim->scene.reversible ? 1 : 0; }

uint32_t dp_sim_kernel(const dp_sim *sim) { return sim ? sim->kernel : 0; }

uint32_t dp_sim_row_pitch(const dp_sim *sim) { return sim ? sim->pitch : 0; }

uint64_t dp_sim_launch_count(const dp_sim *sim) { return sim ? sim->launches : 0; }

} // extern "C"
