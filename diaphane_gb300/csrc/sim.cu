// C ABI: the simulation handle (gpu::Simulation, src/gpu.rs:159-763).
//
// A handle owns its device tables, two field buffer sets and one stream.
// The fused step reads one set and writes the other (ping-pong), which is
// what lets H and E of a whole step be computed in a single pass over HBM.
// The naive passes and the reverse step work in place on the current set.
#include "sim.hpp"

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

namespace {

__global__ void probe_gather(const float *e, const float *h, uint64_t cells, const uint32_t *probe_cells, uint32_t count,
                             float *ring, uint64_t slot) {
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const uint64_t cell = probe_cells[k];
    float *record = ring + (slot * count + k) * 2;
    record[0] = e[2 * cells + cell]; // Ez
    record[1] = h[cells + cell];     // Hy
}

} // namespace

void diaphane::launch_probe_gather(const float *e, const float *h, uint64_t cells, const uint32_t *probe_cells,
                                   uint32_t count, float *ring, uint64_t slot, cudaStream_t stream) {
    probe_gather<<<(count + 127) / 128, 128, 0, stream>>>(e, h, cells, probe_cells, count, ring, slot);
}

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

    uint32_t requested = opts ? opts->kernel : uint32_t(DP_KERNEL_AUTO);
    if (requested > DP_KERNEL_NAIVE) throw Error(DP_ERR_INVALID, "unknown kernel selector");
    // The fused step stages the coefficient table in shared memory and reads
    // a u8 index through its tensor map: at most 256 materials.
    const bool fits = tensor_maps_available() && s.injection_slots() <= size_t(kMaxInjections) && s.index_bytes == 1;
    if (requested == DP_KERNEL_FUSED && !fits)
        throw Error(DP_ERR_UNSUPPORTED, "the fused step takes at most 32 injection slots (2 per source, 8 per "
                                        "total-field box) and 256 materials (and needs the tensor-map encoder)");
    sim->kernel = (requested == DP_KERNEL_NAIVE || !fits) ? DP_KERNEL_NAIVE : DP_KERNEL_FUSED;
    sim->lines = IncidentLines<float>(s);
    if (sim->lines.profile_width()) sim->profile_ring.create(sim->lines.profile_width(), 256);

    DeviceScene &d = sim->dev;
    for (int a = 0; a < 3; ++a) d.n[a] = s.grid.n[a];
    d.pitch = sim->pitch;
    d.cells = cells;
    {
        // The index is rasterized on the device, straight into its buffer.
        uint8_t *material = device_alloc<uint8_t>(cells * s.index_bytes, owned);
        rasterize_on_device(s, material, sim->pitch, st);
        d.material = s.index_bytes == 1 ? material : nullptr;
        d.material16 = s.index_bytes == 2 ? reinterpret_cast<const uint16_t *>(material) : nullptr;
    }
    // Padded to all 256 u8 indices, so a kernel may stage the whole table.
    std::vector<float4> coeff(std::max<size_t>(256, s.coefficients.size()), make_float4(0.0f, 0.0f, 0.0f, 0.0f));
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
            // A plan tuned for this shape earlier in the process, unless the
            // options ask for a particular one.
            const bool defaults = !opts || (opts->cells_per_lane == 0 && opts->tile_y == 0 &&
                                            opts->ring_slots == 0 && opts->z_chunk == 0);
            TunedPlan tuned{};
            if (defaults && tuned_plan(s.grid.n, sms, tuned))
                sim->plan = fused_plan(s.grid.n, tuned.cx, tuned.tile_y, tuned.slots, tuned.z_chunk, sms);
            else
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
        if (sim->scene.has_boxes())
            throw Error(DP_ERR_UNSUPPORTED, "a total-field box's incident line absorbs at its far end, so it does not "
                                            "run backwards");
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
        sim->reset_fields();
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
        if (field != DP_FIELD_INTENSITY) sim->probe_since = sim->step;
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
        sim->probe_since = step;
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

// Not in the public header: raises the error flag a fused step sets when one
// of its bounded waits gives up, so the test suite can check how the host
// reports it without making any wait on the GPU run out.
dp_status dp_internal_raise_wait_error(dp_sim *sim) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        sim->bind();
        const int32_t one = 1;
        check(cudaMemcpyAsync(sim->error, &one, sizeof(one), cudaMemcpyHostToDevice, sim->stream), "error flag");
        check(cudaStreamSynchronize(sim->stream), "error flag");
        return DP_OK;
    });
}

// Not in the public header: sets the fused kernels' plane-wait budget on the
// simulation's device (cycles; negative restores the default, 0 makes every
// plane wait give up at once), so a test can make a wait run out on the GPU
// and watch the kernel report it, drain its loads and exit.
dp_status dp_internal_ring_wait_budget(dp_sim *sim, long long cycles) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        sim->bind();
        check(cudaStreamSynchronize(sim->stream), "ring wait budget");
        try {
            set_ring_wait_budget(cycles);
        } catch (const std::runtime_error &e) {
            throw Error(DP_ERR_CUDA, e.what());
        }
        return DP_OK;
    });
}

dp_status dp_sim_energy_density(dp_sim *sim, float *host, size_t count) {
    return guarded([&] {
        if (!sim || !host) throw Error(DP_ERR_INVALID, "null argument");
        const uint64_t cells = sim->scene.grid.cells();
        if (count != cells) throw Error(DP_ERR_RANGE, "element count does not match the grid");
        sim->bind();
        float *dense = nullptr;
        check(cudaMallocAsync(reinterpret_cast<void **>(&dense), cells * sizeof(float), sim->stream), "density");
        launch_energy_density(sim->dev, sim->fields(), dense, sim->stream);
        ++sim->launches;
        check(cudaGetLastError(), "density launch");
        check(cudaMemcpyAsync(host, dense, cells * sizeof(float), cudaMemcpyDeviceToHost, sim->stream), "density");
        check(cudaFreeAsync(dense, sim->stream), "density");
        sim->wait(kDefaultTimeoutMs);
        return DP_OK;
    });
}

dp_status dp_sim_sample(dp_sim *sim, uint32_t field, uint32_t axis, const uint32_t coord[3], float *out) {
    return guarded([&] {
        if (!sim || !coord || !out) throw Error(DP_ERR_INVALID, "null argument");
        const uint32_t *n = sim->scene.grid.n;
        if (coord[0] >= n[0] || coord[1] >= n[1] || coord[2] >= n[2]) throw Error(DP_ERR_RANGE, "cell outside the grid");
        if (axis > 2 || (field == DP_FIELD_INTENSITY && axis != 0)) throw Error(DP_ERR_RANGE, "no such component");
        const uint64_t at = (uint64_t(coord[2]) * n[1] + coord[1]) * sim->pitch + coord[0];
        const float *src = field_ptr(sim, field) + uint64_t(axis) * sim->padded_cells() + at;
        sim->bind();
        check(cudaMemcpyAsync(out, src, sizeof(float), cudaMemcpyDeviceToHost, sim->stream), "sample");
        sim->wait(kDefaultTimeoutMs);
        return DP_OK;
    });
}

dp_status dp_sim_read_field_async(dp_sim *sim, uint32_t field, float *host, size_t count) {
    return guarded([&] {
        if (!sim || !host) throw Error(DP_ERR_INVALID, "null argument");
        if (count != field_count(sim, field)) throw Error(DP_ERR_RANGE, "element count does not match the field");
        sim->bind();
        sim->copy_out(host, field_ptr(sim, field), field == DP_FIELD_INTENSITY ? 1 : 3);
        return DP_OK;
    });
}

dp_status dp_sim_set_probes(dp_sim *sim, const uint32_t *cells, uint32_t count, uint64_t capacity) {
    return guarded([&] {
        if (!sim || (count && !cells)) throw Error(DP_ERR_INVALID, "null argument");
        if (count && capacity == 0) throw Error(DP_ERR_INVALID, "a probe ring needs room for at least one step");
        // Checked before the byte count is formed, so it cannot wrap.
        if (count && capacity > (uint64_t(1) << 40) / (uint64_t(count) * 2))
            throw Error(DP_ERR_OOM, "a probe ring of more than 2^40 values");
        const uint32_t *n = sim->scene.grid.n;
        std::vector<uint32_t> padded(count);
        for (uint32_t k = 0; k < count; ++k) {
            const uint32_t *c = cells + 3 * k;
            if (c[0] >= n[0] || c[1] >= n[1] || c[2] >= n[2]) throw Error(DP_ERR_RANGE, "probe outside the grid");
            const uint64_t index = (uint64_t(c[2]) * n[1] + c[1]) * sim->pitch + c[0];
            if (index > 0xffffffffull) throw Error(DP_ERR_RANGE, "probe index beyond 32 bits");
            padded[k] = uint32_t(index);
        }
        sim->bind();
        sim->wait(kDefaultTimeoutMs); // the old ring may still be written
        cudaFree(sim->probe_cells);
        cudaFree(sim->probe_ring);
        sim->probe_cells = nullptr;
        sim->probe_ring = nullptr;
        sim->probe_count = 0;
        sim->probe_capacity = 0;
        if (count == 0) return DP_OK;
        check(cudaMalloc(&sim->probe_cells, count * sizeof(uint32_t)), "probe cells");
        check(cudaMalloc(&sim->probe_ring, size_t(capacity) * count * 2 * sizeof(float)), "probe ring");
        check(cudaMemcpy(sim->probe_cells, padded.data(), count * sizeof(uint32_t), cudaMemcpyHostToDevice), "probes");
        sim->probe_count = count;
        sim->probe_capacity = capacity;
        sim->probe_since = sim->step;
        return DP_OK;
    });
}

dp_status dp_sim_read_probes(dp_sim *sim, uint64_t first_step, uint64_t steps, float *host, size_t count) {
    return guarded([&] {
        if (!sim || (steps && !host)) throw Error(DP_ERR_INVALID, "null argument");
        if (count != steps * sim->probe_count * 2) throw Error(DP_ERR_RANGE, "element count does not match the window");
        if (steps == 0) return DP_OK;
        const uint64_t last = first_step + steps - 1;
        const uint64_t oldest = std::max(sim->probe_since + 1, sim->step >= sim->probe_capacity
                                                                   ? sim->step - sim->probe_capacity + 1
                                                                   : uint64_t(1));
        if (first_step < oldest || last > sim->step)
            throw Error(DP_ERR_RANGE, "those steps are not in the probe ring");
        sim->bind();
        sim->wait(kDefaultTimeoutMs);
        const size_t record = size_t(sim->probe_count) * 2;
        uint64_t s = first_step;
        float *out = host;
        while (s <= last) {
            const uint64_t slot = (s - 1) % sim->probe_capacity;
            const uint64_t run = std::min(last - s + 1, sim->probe_capacity - slot);
            check(cudaMemcpy(out, sim->probe_ring + slot * record, run * record * sizeof(float), cudaMemcpyDeviceToHost),
                  "probe readback");
            out += run * record;
            s += run;
        }
        return DP_OK;
    });
}

} // extern "C"
