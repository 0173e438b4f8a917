// C ABI: status strings, grid queries and the resolved host-side scene.
#include "abi.hpp"

#include <cmath>
#include <cstring>

namespace diaphane {

static thread_local std::string g_last_error;

void set_last_error(const std::string &message) { g_last_error = message; }
void clear_last_error() { g_last_error.clear(); }

} // namespace diaphane

struct dp_scene {
    diaphane::Scene scene;
};

using namespace diaphane;

extern "C" {

const char *dp_last_error(void) { return g_last_error.c_str(); }

const char *dp_status_string(dp_status status) {
    switch (status) {
    case DP_OK: return "ok";
    case DP_ERR_INVALID: return "invalid scene or argument";
    case DP_ERR_LOSSY: return "scene is lossy and cannot be reversed";
    case DP_ERR_CUDA: return "CUDA error";
    case DP_ERR_TIMEOUT: return "timed out";
    case DP_ERR_OOM: return "out of memory";
    case DP_ERR_UNSUPPORTED: return "unsupported by this build";
    case DP_ERR_RANGE: return "out of range";
    case DP_ERR_BUSY: return "busy";
    }
    return "unknown status";
}

dp_status dp_grid_resolve(const dp_grid_spec *spec, dp_grid_info *out) {
    return guarded([&] {
        if (!spec || !out) throw Error(DP_ERR_INVALID, "null argument");
        ResolvedGrid g = ResolvedGrid::build(*spec);
        float worst = 1.0f;
        for (int a = 0; a < 3; ++a) {
            out->extent[a] = g.n[a];
            out->size[a] = g.axes[a].length();
            worst = std::fmax(worst, g.axes[a].worst_ratio());
        }
        out->time_step = g.time_step();
        out->finest = g.finest();
        out->coarsest = g.coarsest();
        out->worst_ratio = worst;
        out->reference_cell_size = g.reference_cell_size();
        return DP_OK;
    });
}

dp_status dp_grid_map(const dp_grid_spec *spec, uint32_t op, const float in[3], float out[3]) {
    return guarded([&] {
        if (!spec || !in || !out) throw Error(DP_ERR_INVALID, "null argument");
        ResolvedGrid g = ResolvedGrid::build(*spec);
        switch (op) {
        case DP_MAP_TO_CELL:
            for (int a = 0; a < 3; ++a) out[a] = g.axes[a].coordinate(in[a]);
            break;
        case DP_MAP_TO_POSITION:
            for (int a = 0; a < 3; ++a) out[a] = g.axes[a].position(in[a]);
            break;
        case DP_MAP_CELL_CONTAINING: {
            uint32_t c[3];
            g.cell_containing(in, c);
            for (int a = 0; a < 3; ++a) out[a] = float(c[a]);
            break;
        }
        case DP_MAP_CELL_CENTER: {
            uint32_t c[3];
            for (int a = 0; a < 3; ++a) {
                if (!(in[a] >= 0.0f) || in[a] >= float(g.n[a])) throw Error(DP_ERR_RANGE, "cell outside the grid");
                c[a] = uint32_t(in[a]);
            }
            g.cell_center(c, out);
            break;
        }
        default:
            throw Error(DP_ERR_INVALID, "unknown grid map");
        }
        return DP_OK;
    });
}

dp_status dp_scene_create(const dp_scene_desc *desc, dp_scene **out) {
    return guarded([&] {
        if (!desc || !out) throw Error(DP_ERR_INVALID, "null argument");
        *out = nullptr;
        auto *s = new dp_scene{Scene::build(*desc)};
        *out = s;
        return DP_OK;
    });
}

void dp_scene_destroy(dp_scene *scene) { delete scene; }

dp_status dp_scene_info_get(const dp_scene *scene, dp_scene_info *out) {
    return guarded([&] {
        if (!scene || !out) throw Error(DP_ERR_INVALID, "null argument");
        const Scene &s = scene->scene;
        for (int a = 0; a < 3; ++a) out->extent[a] = s.grid.n[a];
        out->material_count = uint32_t(s.materials.size());
        out->time_step = s.dt;
        out->courant = s.grid.courant;
        out->absorber_peak = s.absorber_peak;
        out->reversible = s.reversible ? 1 : 0;
        out->index_bytes = s.index_bytes;
        return DP_OK;
    });
}

dp_status dp_scene_cell_lookup(const dp_scene *scene, uint32_t samples, float *host, size_t count) {
    return guarded([&] {
        if (!scene || !host) throw Error(DP_ERR_INVALID, "null argument");
        const Scene &s = scene->scene;
        if (samples == 0) samples = s.lookup_samples();
        if (samples < 2) throw Error(DP_ERR_RANGE, "a lookup needs at least two samples per axis");
        if (count != 3 * size_t(samples)) throw Error(DP_ERR_RANGE, "count must be 3 × samples");
        const std::vector<float> lookup = s.cell_lookup(samples);
        std::copy(lookup.begin(), lookup.end(), host);
        return DP_OK;
    });
}

uint32_t dp_scene_lookup_samples(const dp_scene *scene) { return scene ? scene->scene.lookup_samples() : 0; }

dp_status dp_scene_table(const dp_scene *scene, uint32_t table, void *host, size_t bytes) {
    return guarded([&] {
        if (!scene || !host) throw Error(DP_ERR_INVALID, "null argument");
        const Scene &s = scene->scene;
        const void *src = nullptr;
        size_t size = 0;
        switch (table) {
        case DP_TABLE_MAGNETIC_GAINS: src = s.magnetic_gains.data(); size = s.magnetic_gains.size() * 4; break;
        case DP_TABLE_ELECTRIC_GAINS: src = s.electric_gains.data(); size = s.electric_gains.size() * 4; break;
        case DP_TABLE_CELL_CENTERS: src = s.centers.data(); size = s.centers.size() * 4; break;
        case DP_TABLE_ABSORBER: src = s.absorber.data(); size = s.absorber.size() * 4; break;
        case DP_TABLE_COEFFICIENTS: src = s.coefficients.data(); size = s.coefficients.size() * sizeof(Coeff); break;
        case DP_TABLE_MATERIAL_INDEX: src = s.material_index().data(); size = s.material_index().size(); break;
        case DP_TABLE_PRIMARY: src = s.primary.data(); size = s.primary.size() * 4; break;
        case DP_TABLE_DUAL: src = s.dual.data(); size = s.dual.size() * 4; break;
        default: throw Error(DP_ERR_INVALID, "unknown table");
        }
        if (bytes != size) throw Error(DP_ERR_RANGE, "table is " + std::to_string(size) + " bytes");
        std::memcpy(host, src, size);
        return DP_OK;
    });
}

dp_status dp_scene_injections(const dp_scene *scene, float time, dp_injection *out, uint32_t capacity,
                              uint32_t *count) {
    return guarded([&] {
        if (!scene || !count || (capacity && !out)) throw Error(DP_ERR_INVALID, "null argument");
        std::vector<StepInjection> injections;
        scene->scene.injections(time, injections);
        *count = uint32_t(injections.size());
        if (injections.size() > capacity) throw Error(DP_ERR_RANGE, "capacity too small");
        for (size_t i = 0; i < injections.size(); ++i) {
            const StepInjection &s = injections[i];
            dp_injection &o = out[i];
            for (int a = 0; a < 3; ++a) {
                o.origin[a] = s.origin[a];
                o.extent[a] = s.extent[a];
                o.center[a] = s.center[a];
            }
            o.component = s.component;
            o.magnetic = s.magnetic;
            o.value = s.value;
            o.inverse_waist_squared = s.inverse_waist_squared;
        }
        return DP_OK;
    });
}

} // extern "C"

// Internal accessor for the simulation translation unit.
namespace diaphane {
const Scene &scene_of(const dp_scene *s) { return s->scene; }
} // namespace diaphane
