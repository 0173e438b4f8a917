// C ABI: the FP64 instance — the same time step as dp_sim, run in double on
// the GPU with the one-thread-per-cell passes.
//
// Fields, curls, the semi-implicit updates, the drive values and the time are
// double; gains, losses, coefficients and apodization weights are the f32
// setup values promoted (the loss is summed in f32 first, as the tables
// are).  That is the reference's Simulation with T = f64 over f32 setup, the
// arithmetic the f32 step's error is stated against.
#include "abi.hpp"
#include "device.cuh"
#include "profiles.hpp"

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

constexpr uint32_t kTimeoutMs = 600000;

} // namespace

struct dp_sim64 {
    Scene scene;
    int device = 0;
    cudaStream_t stream = nullptr;
    DeviceScene dev{};
    FieldSet64 fields{};
    float *primary = nullptr, *dual = nullptr;
    float2 *eps_mu = nullptr;
    double *partials = nullptr, *host_partials = nullptr;
    std::vector<void *> owned;
    uint64_t step = 0;
    uint64_t launches = 0;
    std::vector<InjectionOf<double>> injections;
    IncidentLines<double> lines; // total-field boxes, in double like the drive
    ProfileRing<double> profile_ring;
    std::vector<double> profile_values;
    const double *step_profiles = nullptr;

    ~dp_sim64() {
        if (stream) {
            cudaSetDevice(device);
            cudaStreamSynchronize(stream);
        }
        for (void *p : owned) cudaFree(p);
        if (host_partials) cudaFreeHost(host_partials);
        if (stream) cudaStreamDestroy(stream);
    }

    void bind() { check(cudaSetDevice(device), "cudaSetDevice"); }

    template <typename T> T *alloc(size_t count) {
        void *p = nullptr;
        check(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)), "cudaMalloc");
        owned.push_back(p);
        return static_cast<T *>(p);
    }
    template <typename T> T *upload(const std::vector<T> &host) {
        T *p = alloc<T>(host.size());
        if (!host.empty())
            check(cudaMemcpyAsync(p, host.data(), host.size() * sizeof(T), cudaMemcpyHostToDevice, stream), "upload");
        return p;
    }

    // apply_sources (src/cpu.rs:606-633) for one phase, in source order.
    void inject_phase(bool magnetic) {
        for (const InjectionOf<double> &s : injections) {
            if (s.value == 0.0 || bool(s.magnetic) != magnetic) continue;
            DeviceInjection d{};
            for (int a = 0; a < 3; ++a) {
                d.origin[a] = s.origin[a];
                d.extent[a] = s.extent[a];
            }
            d.component = s.component;
            d.magnetic = s.magnetic;
            d.weight_offset = s.weight_offset;
            d.profile_offset = s.profile_offset;
            d.profile_axis = s.profile_axis;
            launch_inject(dev, fields, d, s.value, step_profiles, stream);
            ++launches;
        }
    }

    // advance, src/cpu.rs:174-198; the time (step + 1)·dt is exact in f64.
    void forward(uint64_t steps) {
        for (uint64_t n = 0; n < steps; ++n) {
            const double time = double(step + 1) * double(scene.dt);
            const std::vector<BoxCorrections<double>> *boxes = lines.empty() ? nullptr : &lines.at(step);
            scene.injections_in<double>(time, injections, boxes, &profile_values);
            step_profiles = profile_values.empty() ? nullptr : profile_ring.put(profile_values, stream);
            launch_naive_magnetic(dev, fields, false, stream);
            inject_phase(true);
            launch_naive_electric(dev, fields, false, stream);
            inject_phase(false);
            launches += 2;
            check(cudaGetLastError(), "step launch");
            ++step;
        }
    }

    void wait(uint32_t timeout_ms) {
        const cudaError_t q = poll_stream(stream, timeout_ms);
        if (q == cudaErrorNotReady) throw Error(DP_ERR_TIMEOUT, "the GPU did not finish in time");
        check(q, "stream");
    }
};

extern "C" {

dp_status dp_sim64_create(const dp_scene *scene, int32_t device, dp_sim64 **out) {
    return guarded([&] {
        if (!scene || !out) throw Error(DP_ERR_INVALID, "null argument");
        *out = nullptr;
        int count = 0;
        check(cudaGetDeviceCount(&count), "cudaGetDeviceCount");
        if (device < 0 || device >= count) throw Error(DP_ERR_CUDA, "no such CUDA device");
        auto sim = std::make_unique<dp_sim64>();
        sim->scene = scene_of(scene);
        sim->device = device;
        sim->bind();
        check(cudaStreamCreateWithFlags(&sim->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        const Scene &s = sim->scene;
        sim->lines = IncidentLines<double>(s);
        if (sim->lines.profile_width()) sim->profile_ring.create(sim->lines.profile_width(), 256);
        const uint64_t cells = s.grid.cells();
        DeviceScene &d = sim->dev;
        for (int a = 0; a < 3; ++a) d.n[a] = s.grid.n[a];
        d.pitch = s.grid.n[0]; // dense rows: the one-thread-per-cell passes need no padding
        d.cells = cells;
        uint8_t *material = sim->alloc<uint8_t>(cells * s.index_bytes);
        rasterize_on_device(s, material, s.grid.n[0], sim->stream);
        d.material = s.index_bytes == 1 ? material : nullptr;
        d.material16 = s.index_bytes == 2 ? reinterpret_cast<const uint16_t *>(material) : nullptr;
        std::vector<float4> coeff(std::max<size_t>(256, s.coefficients.size()), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        for (size_t m = 0; m < s.coefficients.size(); ++m) {
            const Coeff &c = s.coefficients[m];
            coeff[m] = make_float4(c.electric_gain, c.electric_loss, c.magnetic_gain, c.magnetic_loss);
        }
        d.coeff = sim->upload(coeff);
        d.mgain = sim->upload(s.magnetic_gains);
        d.egain = sim->upload(s.electric_gains);
        d.absorber = sim->upload(s.absorber);
        d.weights = sim->upload(s.weights);
        sim->primary = sim->upload(s.primary);
        sim->dual = sim->upload(s.dual);
        std::vector<float2> eps_mu;
        for (const dp_material &m : s.materials)
            eps_mu.push_back(make_float2(m.relative_permittivity, m.relative_permeability));
        sim->eps_mu = sim->upload(eps_mu);
        sim->fields.e = sim->alloc<double>(3 * cells);
        sim->fields.h = sim->alloc<double>(3 * cells);
        check(cudaMemsetAsync(sim->fields.e, 0, 3 * cells * sizeof(double), sim->stream), "memset");
        check(cudaMemsetAsync(sim->fields.h, 0, 3 * cells * sizeof(double), sim->stream), "memset");
        const uint32_t blocks = energy_blocks(cells);
        sim->partials = sim->alloc<double>(2 * size_t(blocks));
        check(cudaMallocHost(&sim->host_partials, 2 * size_t(blocks) * sizeof(double)), "cudaMallocHost");
        check(cudaStreamSynchronize(sim->stream), "setup upload");
        *out = sim.release();
        return DP_OK;
    });
}

void dp_sim64_destroy(dp_sim64 *sim) { delete sim; }

dp_status dp_sim64_advance(dp_sim64 *sim, uint64_t steps) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        sim->bind();
        sim->forward(steps);
        return DP_OK;
    });
}

dp_status dp_sim64_wait(dp_sim64 *sim, uint32_t timeout_ms) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        sim->bind();
        sim->wait(timeout_ms);
        return DP_OK;
    });
}

uint64_t dp_sim64_step_count(const dp_sim64 *sim) { return sim ? sim->step : 0; }

dp_status dp_sim64_read_field(dp_sim64 *sim, uint32_t field, double *host, size_t count) {
    return guarded([&] {
        if (!sim || !host) throw Error(DP_ERR_INVALID, "null argument");
        if (field != DP_FIELD_ELECTRIC && field != DP_FIELD_MAGNETIC)
            throw Error(DP_ERR_INVALID, "the FP64 instance holds E and H only");
        if (count != 3 * sim->scene.grid.cells()) throw Error(DP_ERR_RANGE, "element count does not match the field");
        sim->bind();
        const double *src = field == DP_FIELD_ELECTRIC ? sim->fields.e : sim->fields.h;
        check(cudaMemcpyAsync(host, src, count * sizeof(double), cudaMemcpyDeviceToHost, sim->stream), "readback");
        sim->wait(kTimeoutMs);
        return DP_OK;
    });
}

dp_status dp_sim64_energy(dp_sim64 *sim, double *electric, double *magnetic) {
    return guarded([&] {
        if (!sim || !electric || !magnetic) throw Error(DP_ERR_INVALID, "null argument");
        sim->bind();
        const uint32_t blocks = energy_blocks(sim->dev.cells);
        launch_energy(sim->dev, sim->fields, sim->primary, sim->dual, sim->eps_mu, sim->partials, blocks, sim->stream);
        ++sim->launches;
        check(cudaGetLastError(), "energy launch");
        check(cudaMemcpyAsync(sim->host_partials, sim->partials, 2 * size_t(blocks) * sizeof(double),
                              cudaMemcpyDeviceToHost, sim->stream),
              "energy readback");
        sim->wait(kTimeoutMs);
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

} // extern "C"
