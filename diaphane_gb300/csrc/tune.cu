// C ABI: autotuning of the fused step for one grid.
//
// The fused kernel comes in several tile shapes (cells per lane × rows per
// tile, with the ring depth each is built with), and a launch splits z into
// chunks whose depth trades start-up work (one rebuilt plane per chunk)
// against how evenly the CTAs fill the GPU.  Which combination is fastest
// depends on the grid's shape and on the scene; dp_sim_autotune times each
// candidate from the simulation's current state on the real workload and
// keeps the fastest.  The state — fields, intensity, step count — is put back
// exactly before every trial and after the last, so tuning changes no result.
#include "sim.hpp"

#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <tuple>

namespace {

// The tuned plans of this process: (nx, ny, nz, SM count) -> plan.
using ShapeKey = std::tuple<uint32_t, uint32_t, uint32_t, int>;
std::mutex g_tuned_mutex;
std::map<ShapeKey, diaphane::TunedPlan> g_tuned;

ShapeKey key_of(const uint32_t n[3], int sms) { return ShapeKey{n[0], n[1], n[2], sms}; }

struct Candidate {
    uint32_t cx, ty, slots, z_chunk;
};

// Fields of the current set and the intensity, saved on the device.
struct Saved {
    float *buffer = nullptr;
    uint64_t step = 0, accumulated = 0;
    int current = 0;
    uint32_t probe_count = 0;

    void save(dp_sim *sim) {
        const uint64_t n = 3 * sim->padded_cells(), cells = sim->padded_cells();
        check_cuda(cudaMallocAsync(reinterpret_cast<void **>(&buffer), (2 * n + cells) * sizeof(float), sim->stream),
                   "tuning scratch");
        const FieldSet f = sim->fields();
        check_cuda(cudaMemcpyAsync(buffer, f.e, n * 4, cudaMemcpyDeviceToDevice, sim->stream), "save");
        check_cuda(cudaMemcpyAsync(buffer + n, f.h, n * 4, cudaMemcpyDeviceToDevice, sim->stream), "save");
        check_cuda(cudaMemcpyAsync(buffer + 2 * n, sim->intensity, cells * 4, cudaMemcpyDeviceToDevice, sim->stream),
                   "save");
        step = sim->step;
        accumulated = sim->accumulated;
        current = sim->current;
        probe_count = sim->probe_count;
    }
    void restore(dp_sim *sim) const {
        const uint64_t n = 3 * sim->padded_cells(), cells = sim->padded_cells();
        sim->current = current;
        const FieldSet f = sim->fields();
        check_cuda(cudaMemcpyAsync(f.e, buffer, n * 4, cudaMemcpyDeviceToDevice, sim->stream), "restore");
        check_cuda(cudaMemcpyAsync(f.h, buffer + n, n * 4, cudaMemcpyDeviceToDevice, sim->stream), "restore");
        check_cuda(cudaMemcpyAsync(sim->intensity, buffer + 2 * n, cells * 4, cudaMemcpyDeviceToDevice, sim->stream),
                   "restore");
        sim->step = step;
        sim->accumulated = accumulated;
    }
    void release(dp_sim *sim) {
        if (buffer) cudaFreeAsync(buffer, sim->stream);
        buffer = nullptr;
    }
};

void use_plan(dp_sim *sim, const FusedPlan &plan) {
    sim->plan = plan;
    try {
        for (int k = 0; k < 2; ++k)
            fused_maps(sim->dev, sim->plan, sim->set[k], sim->material_padded, sim->material_pitch, sim->maps[k]);
    } catch (const std::exception &e) {
        throw Error(DP_ERR_CUDA, e.what());
    }
}

} // namespace

namespace diaphane {

bool tuned_plan(const uint32_t n[3], int sms, TunedPlan &out) {
    std::lock_guard<std::mutex> lock(g_tuned_mutex);
    auto it = g_tuned.find(key_of(n, sms));
    if (it == g_tuned.end()) return false;
    out = it->second;
    return true;
}

void remember_tuned_plan(const uint32_t n[3], int sms, const TunedPlan &plan) {
    std::lock_guard<std::mutex> lock(g_tuned_mutex);
    g_tuned[key_of(n, sms)] = plan;
}

} // namespace diaphane

extern "C" dp_status dp_sim_autotune(dp_sim *sim, uint32_t steps, dp_tuning *out) {
    return guarded([&] {
        if (!sim) throw Error(DP_ERR_INVALID, "null handle");
        dp_tuning result{};
        if (sim->kernel != DP_KERNEL_FUSED) {
            if (out) *out = result; // nothing to tune on the one-thread-per-cell path
            return DP_OK;
        }
        if (steps == 0) steps = 8;
        sim->bind();
        int sms = 0;
        check_cuda(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, sim->device), "attribute");
        const uint32_t *n = sim->scene.grid.n;
        std::vector<Candidate> candidates;
        const Candidate shapes[] = {{4, 8, 3, 0}, {2, 8, 3, 0}, {2, 8, 5, 0}, {4, 16, 3, 0}, {1, 8, 4, 0}, {1, 8, 5, 0}};
        for (const Candidate &shape : shapes) {
            if (!fused_variant_exists(shape.cx, shape.ty, shape.slots)) continue;
            // The wave-filling depth the planner picks (0), and fixed depths.
            for (uint32_t depth : {0u, 16u, 20u, 24u, 32u, 64u, 128u, n[2]}) {
                if (depth > n[2]) continue;
                Candidate c = shape;
                c.z_chunk = depth;
                bool seen = false;
                for (const Candidate &o : candidates)
                    seen = seen || (o.cx == c.cx && o.ty == c.ty && o.slots == c.slots && o.z_chunk == c.z_chunk);
                if (!seen) candidates.push_back(c);
            }
        }
        const FusedPlan original = sim->plan;
        Saved saved;
        saved.save(sim);
        sim->probe_count = 0; // trials record nothing
        cudaEvent_t start = nullptr, stop = nullptr;
        check_cuda(cudaEventCreate(&start), "event");
        check_cuda(cudaEventCreate(&stop), "event");
        float best_ms = 0.0f;
        FusedPlan best = original;
        uint32_t tried = 0;
        try {
            for (const Candidate &c : candidates) {
                FusedPlan plan;
                try {
                    plan = fused_plan(n, c.cx, c.ty, c.slots, c.z_chunk, sms);
                } catch (const std::exception &) {
                    continue;
                }
                use_plan(sim, plan);
                saved.restore(sim);
                sim->forward(2); // warm: first launch of a variant configures it
                saved.restore(sim);
                check_cuda(cudaEventRecord(start, sim->stream), "event");
                sim->forward(steps);
                check_cuda(cudaEventRecord(stop, sim->stream), "event");
                sim->wait(600000);
                float ms = 0.0f;
                check_cuda(cudaEventElapsedTime(&ms, start, stop), "event");
                ms /= float(steps);
                ++tried;
                if (tried == 1 || ms < best_ms) {
                    best_ms = ms;
                    best = plan;
                }
            }
        } catch (...) {
            use_plan(sim, original);
            saved.restore(sim);
            sim->probe_count = saved.probe_count;
            saved.release(sim);
            cudaEventDestroy(start);
            cudaEventDestroy(stop);
            throw;
        }
        use_plan(sim, best);
        saved.restore(sim);
        sim->probe_count = saved.probe_count;
        saved.release(sim);
        sim->wait(600000);
        cudaEventDestroy(start);
        cudaEventDestroy(stop);
        result.cells_per_lane = best.cx;
        result.tile_y = best.tile_y;
        result.ring_slots = best.slots;
        result.z_chunk = best.z_chunk;
        result.ms_per_step = best_ms;
        result.candidates = tried;
        if (tried) remember_tuned_plan(n, sms, TunedPlan{best.cx, best.tile_y, best.slots, best.z_chunk, best_ms});
        if (out) *out = result;
        return DP_OK;
    });
}

extern "C" dp_status dp_sim_plan(const dp_sim *sim, dp_tuning *out) {
    return guarded([&] {
        if (!sim || !out) throw Error(DP_ERR_INVALID, "null argument");
        dp_tuning t{};
        if (sim->kernel == DP_KERNEL_FUSED) {
            t.cells_per_lane = sim->plan.cx;
            t.tile_y = sim->plan.tile_y;
            t.ring_slots = sim->plan.slots;
            t.z_chunk = sim->plan.z_chunk;
        }
        *out = t;
        return DP_OK;
    });
}

// One line per shape: "nx ny nz sms cx tile_y slots z_chunk ms_per_step".
extern "C" dp_status dp_tune_cache_export(char *buf, size_t cap, size_t *len) {
    return guarded([&] {
        if (!len || (cap && !buf)) throw Error(DP_ERR_INVALID, "null argument");
        std::ostringstream text;
        {
            std::lock_guard<std::mutex> lock(g_tuned_mutex);
            for (const auto &kv : g_tuned) {
                const TunedPlan &p = kv.second;
                char line[160];
                std::snprintf(line, sizeof(line), "%u %u %u %d %u %u %u %u %.6g\n", std::get<0>(kv.first),
                              std::get<1>(kv.first), std::get<2>(kv.first), std::get<3>(kv.first), p.cx, p.tile_y,
                              p.slots, p.z_chunk, double(p.ms_per_step));
                text << line;
            }
        }
        const std::string t = text.str();
        *len = t.size();
        if (cap < t.size() + 1) throw Error(DP_ERR_RANGE, "the buffer cannot hold the cache");
        std::memcpy(buf, t.c_str(), t.size() + 1);
        return DP_OK;
    });
}

extern "C" dp_status dp_tune_cache_import(const char *text) {
    return guarded([&] {
        if (!text) throw Error(DP_ERR_INVALID, "null argument");
        std::istringstream in(text);
        std::string line;
        while (std::getline(in, line)) {
            if (line.find_first_not_of(" \t\r") == std::string::npos) continue;
            uint32_t n[3], cx, ty, slots, depth;
            int sms;
            float ms;
            char extra;
            if (std::sscanf(line.c_str(), "%u %u %u %d %u %u %u %u %f %c", &n[0], &n[1], &n[2], &sms, &cx, &ty,
                            &slots, &depth, &ms, &extra) != 9 ||
                !fused_variant_exists(cx, ty, slots) || n[0] == 0 || n[1] == 0 || n[2] == 0 || depth > n[2])
                throw Error(DP_ERR_INVALID, "malformed tuning line: " + line);
            remember_tuned_plan(n, sms, TunedPlan{cx, ty, slots, depth, ms});
        }
        return DP_OK;
    });
}

extern "C" void dp_tune_cache_clear(void) {
    std::lock_guard<std::mutex> lock(g_tuned_mutex);
    g_tuned.clear();
}
