// The batched form: many scenes of uneven sizes advanced together.
//
// Every scene lives in one device arena (fields, intensity, padded material
// index, tables), admitted by bytes against the arena's capacity.  A step of
// the whole batch is one launch per kernel variant over a work list of
// (scene, tile, z-chunk) units drawn from all scenes; a chunk of K steps is
// captured once into a CUDA graph and replayed while the batch's membership
// is unchanged.  What changes from chunk to chunk — each scene's injections
// for each step, how many steps it takes, which field set is current — lives
// in device tables the host rewrites before each replay, so the graph's
// topology never depends on scene content.  Scenes join and leave only
// between chunks; a scene that finishes mid-chunk sits out the rest of it.
#include "abi.hpp"
#include "device.cuh"

#include <algorithm>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <map>
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

constexpr size_t kAlign = 256;

size_t round_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// First-fit allocator over the arena's byte range.
class Arena {
  public:
    void reset(size_t capacity) {
        free_.clear();
        free_[0] = capacity;
        used_ = 0;
        capacity_ = capacity;
    }
    bool allocate(size_t bytes, size_t &offset) {
        if (bytes > SIZE_MAX - kAlign) return false;
        bytes = round_up(bytes, kAlign);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                offset = it->first;
                const size_t rest = it->second - bytes;
                free_.erase(it);
                if (rest) free_[offset + bytes] = rest;
                used_ += bytes;
                return true;
            }
        }
        return false;
    }
    void release(size_t offset, size_t bytes) {
        bytes = round_up(bytes, kAlign);
        used_ -= bytes;
        auto next = free_.lower_bound(offset);
        if (next != free_.end() && offset + bytes == next->first) {
            bytes += next->second;
            next = free_.erase(next);
        }
        if (next != free_.begin()) {
            auto prev = std::prev(next);
            if (prev->first + prev->second == offset) {
                prev->second += bytes;
                return;
            }
        }
        free_[offset] = bytes;
    }
    size_t used() const { return used_; }
    size_t capacity() const { return capacity_; }

  private:
    std::map<size_t, size_t> free_;
    size_t used_ = 0, capacity_ = 0;
};

struct Variant {
    uint32_t cx, tile_y, slots;
    uint32_t scene_x = 0; // stored axis holding the scenes' x
    bool operator==(const Variant &o) const {
        return cx == o.cx && tile_y == o.tile_y && slots == o.slots && scene_x == o.scene_x;
    }
};

// The variant a grid shape runs: the requested tile width, or else the widest
// tile that wastes no more lanes than a narrower one; 8 rows, and the ring
// depth that variant is built with (3 slots for 128- and 64-wide tiles, 4 for
// 32-wide ones, the depths that let 2, 3 and 4 CTAs share an SM).
Variant variant_for(uint32_t nx, uint32_t requested_cx) {
    uint32_t best = 4, waste_best = ~0u;
    for (uint32_t cx : {4u, 2u, 1u}) {
        const uint32_t tx = 32 * cx, waste = (nx + tx - 1) / tx * tx - nx;
        if (waste < waste_best) {
            best = cx;
            waste_best = waste;
        }
    }
    if (requested_cx) best = requested_cx;
    return Variant{best, 8, best == 1 ? 4u : 3u};
}

// A scene's extents in axis order `order`: stored[i] = n[kBatchAxisOrders[order][i]].
void stored_extent(const uint32_t n[3], uint32_t order, uint32_t out[3]) {
    for (int i = 0; i < 3; ++i) out[i] = n[kBatchAxisOrders[order][i]];
}

// The stored axis holding scene axis a (the inverse of kBatchAxisOrders).
uint32_t stored_axis(uint32_t order, uint32_t a) {
    for (uint32_t i = 0; i < 3; ++i)
        if (uint32_t(kBatchAxisOrders[order][i]) == a) return i;
    return a;
}

// The odd permutations, whose scenes keep their gain tables negated.
bool reverses_curls(uint32_t order) { return order >= 1 && order <= 3; }

// The variant a scene stored in axis order `order` runs (stored extents
// `m`): as variant_for, except that a scene whose x is not stored along x
// takes 32-wide tiles, the only ones built to group its loss by the scene's
// axes.
Variant variant_in(const uint32_t m[3], uint32_t order, uint32_t requested_cx) {
    const uint32_t scene_x = stored_axis(order, 0);
    if (scene_x == 0) return variant_for(m[0], requested_cx);
    Variant v = variant_for(m[0], 1);
    v.scene_x = scene_x;
    return v;
}

// Whether a requested tile width (0: none) allows axis order `order`.
bool order_allowed(uint32_t order, uint32_t requested_cx) {
    return stored_axis(order, 0) == 0 || requested_cx == 0 || requested_cx == 1;
}

// Cells a scene's units cover in axis order `order`: whole tiles of the
// variant's width along x and of 8 rows along y, every plane along z;
// UINT64_MAX when the order is ruled out.
uint64_t tiled_cells(const uint32_t n[3], uint32_t order, uint32_t requested_cx) {
    if (!order_allowed(order, requested_cx)) return UINT64_MAX;
    uint32_t m[3];
    stored_extent(n, order, m);
    const uint32_t tx = 32 * variant_in(m, order, requested_cx).cx;
    return uint64_t((m[0] + tx - 1) / tx * tx) * ((m[1] + 7) / 8 * 8) * m[2];
}

// Whether a scene may be stored with its axes permuted: not when a source
// carries apodization weights or a total-field box's side-face profiles,
// which are laid out along the scene's own axes.
bool permutable(const Scene &s) { return s.weights.empty() && !s.has_boxes(); }

// The axis order a scene is stored in.  `requested` 0: the order whose tiles
// cover the fewest cells (ties to the lower order; on 256 mixed scenes with
// axes of 32-160 cells this covers 14 % fewer cells than the scenes' own
// order); k in 1-6: order k-1 for every permutable scene, unless a requested
// tile width rules it out.  The arithmetic does not depend on the order (the
// kernel keeps the scene's operation order), so neither do the results.
uint32_t order_for(const Scene &s, uint32_t requested, uint32_t requested_cx) {
    if (!permutable(s)) return 0;
    if (requested) return order_allowed(requested - 1, requested_cx) ? requested - 1 : 0;
    uint32_t best = 0;
    uint64_t cells_best = tiled_cells(s.grid.n, 0, requested_cx);
    for (uint32_t order = 1; order < 6; ++order) {
        const uint64_t cells = tiled_cells(s.grid.n, order, requested_cx);
        if (cells < cells_best) {
            best = order;
            cells_best = cells;
        }
    }
    return best;
}

struct Entry {
    uint64_t id = 0;
    Scene scene;
    uint32_t slot = 0;            // index into the descriptor array
    Variant variant{};
    uint32_t order = 0;           // axis order the scene is stored in
    uint32_t n[3] = {0, 0, 0};    // its extents in that order
    uint32_t pitch = 0, material_pitch = 0;
    uint64_t cells_padded = 0;
    size_t offset = 0, bytes = 0; // arena block
    BatchScene desc{};
    uint64_t step = 0;            // steps completed
    uint64_t target = 0;          // steps requested
    bool accumulate = false;
    std::vector<uint32_t> probe_cells; // padded linear cell index per probe
    float *probes = nullptr;      // target × probes × 2 (Ez, Hy)
    std::vector<BatchUnit> units;
    IncidentLines<float> lines;   // the scene's total-field boxes, if any
    uint64_t joined = 0;          // chunks the batch had started when the scene joined
    dp_status fault = DP_OK;      // DP_ERR_NONFINITE once a check found a NaN or infinity
};

// Per-step probe gather: after step t of a chunk, Ez and Hy at every probe
// of every scene still stepping.
struct ProbeSlot {
    uint32_t slot;      // scene descriptor index
    uint32_t k;         // probe number within the scene
    uint32_t probes;    // probes of that scene
    uint32_t cell;      // padded linear index, in the scene's stored order
    uint32_t ez, hy;    // the stored components holding the scene's Ez and Hy
    float *series;      // the scene's probe series
};

__global__ void gather_probes(const BatchScene *scenes, const ProbeSlot *slots, uint32_t count, uint32_t step) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const ProbeSlot ps = slots[i];
    const BatchScene &bs = scenes[ps.slot];
    if (step >= bs.steps) return;
    const uint32_t out = (bs.parity + step + 1u) & 1u; // the set this step wrote
    const float ez = bs.e[out][ps.ez * bs.s.cells + ps.cell];
    const float hy = bs.h[out][ps.hy * bs.s.cells + ps.cell];
    const uint64_t at = ((bs.step0 + step) * ps.probes + ps.k) * 2;
    ps.series[at] = ez;
    ps.series[at + 1] = hy;
}

// is_finite (src/cpu.rs:707-713), per scene, after a chunk: one block per
// work unit of one variant (tiles `tx` cells wide, 8 rows) reads the unit's
// cells of all six components in the set the chunk left current and marks
// the scene's slot when any of them is NaN or infinite.  A mark stays set
// until the slot is given to another scene.
__global__ void scan_finite(const BatchScene *scenes, const BatchUnit *units, uint32_t tx, int32_t *marks) {
    const BatchUnit unit = units[blockIdx.x];
    const BatchScene &bs = scenes[unit.scene];
    if (bs.steps == 0) return;
    const uint32_t set = (bs.parity + bs.steps) & 1u;
    const uint32_t ny = bs.s.n[1];
    const uint32_t width = min(tx, bs.s.n[0] - unit.x0), rows = min(8u, ny - unit.y0);
    // Threads run along x (tx of them per row, coalesced); a block covers
    // blockDim / tx rows at a time.  No early exit, so the loads of several
    // planes are in flight at once.
    const uint32_t x = threadIdx.x % tx, step = blockDim.x / tx;
    const uint64_t pitch = bs.s.pitch;
    bool bad = false;
    if (x < width)
        for (uint32_t c = 0; c < 6; ++c) {
            const float *f = (c < 3 ? bs.e[set] + uint64_t(c) * bs.s.cells : bs.h[set] + uint64_t(c - 3) * bs.s.cells) +
                             unit.x0 + x;
            for (uint32_t yy = threadIdx.x / tx; yy < rows; yy += step) {
                const float *line = f + (uint64_t(unit.z0) * ny + unit.y0 + yy) * pitch;
                const uint64_t plane = uint64_t(ny) * pitch;
#pragma unroll 4
                for (uint32_t z = 0; z < unit.z1 - unit.z0; ++z) bad |= !isfinite(__ldcs(line + z * plane));
            }
        }
    if (__syncthreads_or(bad) && threadIdx.x == 0) marks[unit.scene] = 1;
}

// Scene coordinates of stored cell (x, y, z) in an axis order: the scene's
// coordinate along axes.a[i] is the stored coordinate i.
struct Axes {
    uint32_t a[3];
};

// The material index in a scene's stored axis order, rows of out_pitch cells
// (past the stored x extent: 0), from the scene's own index (rows of
// in_pitch).  One thread per stored cell.
__global__ void index_to_stored(const uint8_t *in, uint32_t in_pitch, uint32_t scene_ny, uint8_t *out,
                                uint32_t out_pitch, uint32_t nx, uint32_t ny, uint64_t total, Axes axes) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const uint32_t x = uint32_t(i % out_pitch);
    const uint64_t r = i / out_pitch;
    const uint32_t y = uint32_t(r % ny), z = uint32_t(r / ny);
    uint8_t v = 0;
    if (x < nx) {
        uint32_t q[3];
        q[axes.a[0]] = x;
        q[axes.a[1]] = y;
        q[axes.a[2]] = z;
        v = in[(uint64_t(q[2]) * scene_ny + q[1]) * in_pitch + q[0]];
    }
    out[i] = v;
}

// A stored field back in the scene's own order, dense: component c of scene
// cell (x, y, z) is stored component comp.a[c] at the stored cell whose
// coordinate i is the scene's coordinate along axes.a[i].  One thread per
// output value.
__global__ void field_from_stored(const float *stored, uint64_t stride, uint32_t pitch, uint32_t stored_ny, Axes axes,
                                  Axes comp, uint32_t nx, uint32_t ny, uint64_t cells, uint64_t total, float *out) {
    const uint64_t i = uint64_t(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= total) return;
    const uint32_t c = uint32_t(i / cells);
    const uint64_t cell = i % cells;
    uint32_t q[3];
    q[0] = uint32_t(cell % nx);
    q[1] = uint32_t((cell / nx) % ny);
    q[2] = uint32_t(cell / (uint64_t(nx) * ny));
    const uint64_t at = (uint64_t(q[axes.a[2]]) * stored_ny + q[axes.a[1]]) * pitch + q[axes.a[0]];
    out[i] = stored[comp.a[c] * stride + at];
}

Axes axes_of(uint32_t order) {
    Axes a{};
    for (int i = 0; i < 3; ++i) a.a[i] = uint32_t(kBatchAxisOrders[order][i]);
    return a;
}

void make_units(Entry &e, uint32_t planes);

} // namespace

struct dp_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    uint32_t chunk = 50;
    uint32_t capacity = 0;        // scene slots
    uint32_t cells_per_lane = 0;  // forced tile width (0: per scene)
    uint32_t axis_order = 0;      // forced axis order + 1 (0: per scene)
    uint32_t unit_planes = 24;    // z-planes per work unit
    bool unit_planes_set = false; // configured, rather than chosen per rebuild
    int sm_count = 1;
    bool graphs = true;
    unsigned char *arena_base = nullptr;
    Arena arena;
    std::map<uint64_t, Entry> entries;
    std::vector<int> slot_used;
    uint64_t next_id = 1;
    // Device tables.
    BatchScene *scenes = nullptr;                 // [capacity]
    DeviceInjection *injections = nullptr;        // [2][chunk][capacity][kBatchInjections]
    uint32_t *counts = nullptr;                   // [2][chunk][capacity]
    std::vector<BatchUnit *> units;               // per variant
    std::vector<uint32_t> unit_counts;
    std::vector<Variant> variants;
    ProbeSlot *probe_slots = nullptr;             // grouped by variant
    uint32_t probe_count = 0;
    std::vector<uint32_t> probe_offset, probe_count_v; // each variant's share of probe_slots
    // One stream per variant: the variants' scenes are disjoint, so within a
    // chunk their launches form independent chains that may overlap.
    std::vector<cudaStream_t> lanes;
    std::vector<cudaEvent_t> joins;
    cudaEvent_t fork = nullptr;
    int32_t *error = nullptr;
    // Non-finite marks per slot (device), copied after every chunk into the
    // pinned area of that chunk's staging half, with the event that says the
    // copy has landed and the number of the chunk it belongs to.
    bool check_finite = true;
    int32_t *marks = nullptr;
    int32_t *h_marks[2] = {nullptr, nullptr};
    cudaEvent_t marked[2] = {nullptr, nullptr};
    bool marks_pending[2] = {false, false};
    uint64_t marks_chunk[2] = {0, 0};
    // Host staging (pinned), double-buffered against in-flight copies.
    BatchScene *h_scenes[2] = {nullptr, nullptr};
    DeviceInjection *h_injections[2] = {nullptr, nullptr};
    uint32_t *h_counts[2] = {nullptr, nullptr};
    // Total-field boxes' side-face values of one chunk, per staging half:
    // every box scene's steps back to back, indexed by its injections.
    float *profiles = nullptr;                    // [2][profile_capacity] device
    float *h_profiles[2] = {nullptr, nullptr};    // pinned
    size_t profile_capacity = 0;
    cudaEvent_t staged[2] = {nullptr, nullptr};
    int stage = 0;
    // Graph of one chunk, rebuilt when the work lists change.
    bool dirty = true;
    cudaGraphExec_t exec[2] = {nullptr, nullptr}; // one per staging half
    uint64_t launches = 0;
    uint64_t chunks_run = 0;

    void bind() { check(cudaSetDevice(device), "cudaSetDevice"); }

    ~dp_batch() {
        if (stream) {
            cudaSetDevice(device);
            cudaStreamSynchronize(stream);
        }
        for (auto &e : exec)
            if (e) cudaGraphExecDestroy(e);
        for (BatchUnit *u : units) cudaFree(u);
        cudaFree(scenes);
        cudaFree(injections);
        cudaFree(counts);
        cudaFree(probe_slots);
        cudaFree(error);
        cudaFree(marks);
        for (cudaStream_t l : lanes) cudaStreamDestroy(l);
        for (cudaEvent_t e : joins) cudaEventDestroy(e);
        if (fork) cudaEventDestroy(fork);
        cudaFree(arena_base);
        cudaFree(profiles);
        for (int k = 0; k < 2; ++k) {
            cudaFreeHost(h_profiles[k]);
            cudaFreeHost(h_scenes[k]);
            cudaFreeHost(h_injections[k]);
            cudaFreeHost(h_counts[k]);
            cudaFreeHost(h_marks[k]);
            if (staged[k]) cudaEventDestroy(staged[k]);
            if (marked[k]) cudaEventDestroy(marked[k]);
        }
        if (stream) cudaStreamDestroy(stream);
    }

    size_t injection_span() const { return size_t(chunk) * capacity * kBatchInjections; }
    size_t count_span() const { return size_t(chunk) * capacity; }

    // Work lists and probe slots from the current membership.
    void rebuild_lists() {
        // The previous chunk may still be reading the old lists.
        check(cudaStreamSynchronize(stream), "previous chunk");
        for (BatchUnit *u : units) cudaFree(u);
        units.clear();
        unit_counts.clear();
        variants.clear();
        // Unit depth: the configured one; else 64 planes when the batch holds
        // enough work to fill many waves with units that deep (fewer rebuilt
        // planes and CTA start-ups: 2 % faster on 256 mixed scenes), and 24
        // otherwise, so that a lightly loaded batch still spreads each scene
        // over the GPU.
        uint32_t depth = unit_planes;
        if (!unit_planes_set) {
            uint64_t deep_units = 0;
            for (auto &kv : entries) {
                const uint32_t *n = kv.second.n;
                const uint32_t tx = 32 * kv.second.variant.cx, ty = kv.second.variant.tile_y;
                deep_units += uint64_t((n[0] + tx - 1) / tx) * ((n[1] + ty - 1) / ty) * ((n[2] + 63) / 64);
            }
            if (deep_units >= 16ull * uint64_t(sm_count)) depth = 64;
        }
        for (auto &kv : entries) make_units(kv.second, depth);
        // Room for a whole chunk of every box scene's side-face values (the
        // stream is idle here, so the old buffers can go).
        size_t profile_need = 0;
        for (auto &kv : entries) profile_need += size_t(chunk) * kv.second.lines.profile_width();
        if (profile_need > profile_capacity) {
            cudaFree(profiles);
            profiles = nullptr;
            for (auto &hp : h_profiles) {
                cudaFreeHost(hp);
                hp = nullptr;
            }
            profile_capacity = 0;
            check(cudaMalloc(&profiles, 2 * profile_need * sizeof(float)), "cudaMalloc profiles");
            for (auto &hp : h_profiles) check(cudaMallocHost(&hp, profile_need * sizeof(float)), "profile staging");
            profile_capacity = profile_need;
        }
        std::vector<std::vector<BatchUnit>> lists;
        std::vector<std::vector<ProbeSlot>> probe_lists;
        for (auto &kv : entries) {
            Entry &e = kv.second;
            size_t v = 0;
            while (v < variants.size() && !(variants[v] == e.variant)) ++v;
            if (v == variants.size()) {
                variants.push_back(e.variant);
                lists.emplace_back();
                probe_lists.emplace_back();
            }
            lists[v].insert(lists[v].end(), e.units.begin(), e.units.end());
            for (uint32_t k = 0; k < e.probe_cells.size(); ++k)
                probe_lists[v].push_back(ProbeSlot{e.slot, k, uint32_t(e.probe_cells.size()), e.probe_cells[k],
                                                   stored_axis(e.order, 2), stored_axis(e.order, 1), e.probes});
        }
        std::vector<ProbeSlot> probes;
        probe_offset.clear();
        probe_count_v.clear();
        for (auto &pl : probe_lists) {
            probe_offset.push_back(uint32_t(probes.size()));
            probe_count_v.push_back(uint32_t(pl.size()));
            probes.insert(probes.end(), pl.begin(), pl.end());
        }
        while (lanes.size() < variants.size()) {
            cudaStream_t l = nullptr;
            cudaEvent_t j = nullptr;
            check(cudaStreamCreateWithFlags(&l, cudaStreamNonBlocking), "lane stream");
            check(cudaEventCreateWithFlags(&j, cudaEventDisableTiming), "lane event");
            lanes.push_back(l);
            joins.push_back(j);
        }
        if (!fork) check(cudaEventCreateWithFlags(&fork, cudaEventDisableTiming), "fork event");
        for (auto &list : lists) {
            BatchUnit *d = nullptr;
            check(cudaMalloc(&d, std::max<size_t>(1, list.size()) * sizeof(BatchUnit)), "cudaMalloc units");
            check(cudaMemcpyAsync(d, list.data(), list.size() * sizeof(BatchUnit), cudaMemcpyHostToDevice, stream),
                  "units");
            units.push_back(d);
            unit_counts.push_back(uint32_t(list.size()));
        }
        cudaFree(probe_slots);
        probe_slots = nullptr;
        probe_count = uint32_t(probes.size());
        check(cudaMalloc(&probe_slots, std::max<size_t>(1, probes.size()) * sizeof(ProbeSlot)), "cudaMalloc probes");
        if (!probes.empty())
            check(cudaMemcpyAsync(probe_slots, probes.data(), probes.size() * sizeof(ProbeSlot),
                                  cudaMemcpyHostToDevice, stream),
                  "probe slots");
        check(cudaStreamSynchronize(stream), "work lists");
        for (auto &x : exec)
            if (x) {
                cudaGraphExecDestroy(x);
                x = nullptr;
            }
        dirty = false;
    }

    // The launches of one chunk reading staging half `half`: one chain per
    // variant (its steps and its scenes' probe gathers, in order) on that
    // variant's stream, forked from and joined back into the batch stream.
    void record_chunk(int half) {
        const DeviceInjection *inj = injections + size_t(half) * injection_span();
        const uint32_t *cnt = counts + size_t(half) * count_span();
        const float *prof = profiles ? profiles + size_t(half) * profile_capacity : nullptr;
        check(cudaEventRecord(fork, stream), "fork");
        for (size_t v = 0; v < variants.size(); ++v) {
            cudaStream_t lane = lanes[v];
            check(cudaStreamWaitEvent(lane, fork, 0), "fork");
            for (uint32_t t = 0; t < chunk; ++t) {
                launch_batch_step(variants[v].cx, variants[v].tile_y, variants[v].slots, variants[v].scene_x,
                                  scenes, units[v], unit_counts[v], inj, cnt, prof, capacity, t, error, lane);
                ++launches;
                if (probe_count_v[v]) {
                    gather_probes<<<(probe_count_v[v] + 255) / 256, 256, 0, lane>>>(
                        scenes, probe_slots + probe_offset[v], probe_count_v[v], t);
                    ++launches;
                }
            }
            if (check_finite && unit_counts[v]) {
                scan_finite<<<unit_counts[v], 256, 0, lane>>>(scenes, units[v], 32 * variants[v].cx, marks);
                ++launches;
            }
            check(cudaEventRecord(joins[v], lane), "join");
            check(cudaStreamWaitEvent(stream, joins[v], 0), "join");
        }
        if (check_finite)
            check(cudaMemcpyAsync(h_marks[half], marks, size_t(capacity) * sizeof(int32_t), cudaMemcpyDeviceToHost,
                                  stream),
                  "finite marks");
    }

    // Applies the marks of finished chunks: a scene found non-finite stops
    // stepping (its target becomes the steps issued for it) and reports
    // DP_ERR_NONFINITE; the others run on untouched, each scene's arithmetic
    // being its own.  `wait_half` (0 or 1) is waited for, the other half only
    // taken when its copy has already landed; -1 waits for both, -2 for
    // neither.
    void collect_marks(int wait_half) {
        for (int half = 0; half < 2; ++half) {
            if (!marks_pending[half]) continue;
            if (wait_half == -1 || half == wait_half) {
                check(cudaEventSynchronize(marked[half]), "finite marks");
            } else {
                const cudaError_t q = cudaEventQuery(marked[half]);
                if (q == cudaErrorNotReady) continue;
                check(q, "finite marks");
            }
            marks_pending[half] = false;
            for (auto &kv : entries) {
                Entry &e = kv.second;
                if (e.fault != DP_OK || e.joined > marks_chunk[half] || !h_marks[half][e.slot]) continue;
                e.fault = DP_ERR_NONFINITE;
                e.target = e.step;
            }
        }
    }

    // One chunk: stage descriptors and injections, then replay (or launch).
    uint32_t run_chunk() {
        // The marks of the chunk two back (whose staging half this one
        // reuses) are waited for, so a scene that turned non-finite stops
        // within two chunks; the chunk in between keeps the GPU busy.
        collect_marks(stage);
        // A chunk right after a membership change launches directly: a graph
        // pays off only once it is replayed, and membership that changes
        // every chunk (requests arriving and leaving) would never replay one.
        const bool changed = dirty;
        if (dirty) rebuild_lists();
        const int half = stage;
        // The staging half is free once the copies that last read it are done.
        check(cudaEventSynchronize(staged[half]), "staging");
        BatchScene *hs = h_scenes[half];
        DeviceInjection *hi = h_injections[half];
        uint32_t *hc = h_counts[half];
        std::memset(hc, 0, count_span() * sizeof(uint32_t));
        uint32_t stepping = 0;
        std::vector<StepInjection> step_injections;
        std::vector<float> step_profiles;
        size_t profile_cursor = 0;
        float *hp = h_profiles[half];
        std::vector<ProbeSlot> probe_updates;
        for (auto &kv : entries) {
            Entry &e = kv.second;
            const uint64_t remaining = e.target > e.step ? e.target - e.step : 0;
            const uint32_t steps = uint32_t(std::min<uint64_t>(remaining, chunk));
            e.desc.steps = steps;
            e.desc.parity = uint32_t(e.step & 1u);
            e.desc.step0 = e.step;
            hs[e.slot] = e.desc;
            if (steps) ++stepping;
            for (uint32_t t = 0; t < steps; ++t) {
                const float time = float(e.step + t + 1) * e.scene.dt;
                int32_t rebase = 0;
                if (e.lines.empty()) {
                    e.scene.injections(time, step_injections);
                } else {
                    e.scene.injections_in<float>(time, step_injections, &e.lines.at(e.step + t), &step_profiles);
                    if (profile_cursor + step_profiles.size() > profile_capacity)
                        throw Error(DP_ERR_CUDA, "box profiles exceed the batch's staging");
                    std::memcpy(hp + profile_cursor, step_profiles.data(), step_profiles.size() * sizeof(float));
                    rebase = int32_t(profile_cursor);
                    profile_cursor += step_profiles.size();
                }
                uint32_t n = 0;
                DeviceInjection *row = hi + (size_t(t) * capacity + e.slot) * kBatchInjections;
                for (const StepInjection &si : step_injections) {
                    if (si.value == 0.0f) continue;
                    if (n == kBatchInjections) throw Error(DP_ERR_UNSUPPORTED, "too many injections for a batch scene");
                    // In the scene's stored axis order (a permuted scene
                    // has neither weights nor box profiles).
                    DeviceInjection &d = row[n++];
                    const int *axes = kBatchAxisOrders[e.order];
                    for (int i = 0; i < 3; ++i) {
                        d.origin[i] = si.origin[axes[i]];
                        d.extent[i] = si.extent[axes[i]];
                    }
                    d.component = stored_axis(e.order, si.component);
                    d.magnetic = si.magnetic;
                    d.value = si.value;
                    d.weight_offset = si.weight_offset;
                    d.profile_offset = si.profile_offset < 0 ? -1 : si.profile_offset + rebase;
                    d.profile_axis = stored_axis(e.order, si.profile_axis);
                }
                hc[size_t(t) * capacity + e.slot] = n;
            }
        }
        check(cudaMemcpyAsync(scenes, hs, size_t(capacity) * sizeof(BatchScene), cudaMemcpyHostToDevice, stream),
              "descriptors");
        check(cudaMemcpyAsync(injections + size_t(half) * injection_span(), hi,
                              injection_span() * sizeof(DeviceInjection), cudaMemcpyHostToDevice, stream),
              "injections");
        check(cudaMemcpyAsync(counts + size_t(half) * count_span(), hc, count_span() * sizeof(uint32_t),
                              cudaMemcpyHostToDevice, stream),
              "counts");
        if (profile_cursor)
            check(cudaMemcpyAsync(profiles + size_t(half) * profile_capacity, hp, profile_cursor * sizeof(float),
                                  cudaMemcpyHostToDevice, stream),
                  "profiles");
        check(cudaEventRecord(staged[half], stream), "staging event");
        if (stepping) {
            if (graphs && !changed) {
                if (!exec[half]) {
                    cudaGraph_t graph = nullptr;
                    check(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal), "capture");
                    const uint64_t before = launches;
                    record_chunk(half);
                    check(cudaStreamEndCapture(stream, &graph), "capture");
                    launches = before;
                    check(cudaGraphInstantiate(&exec[half], graph, 0), "instantiate");
                    cudaGraphDestroy(graph);
                }
                check(cudaGraphLaunch(exec[half], stream), "graph launch");
                uint64_t per_step = variants.size();
                for (uint32_t c : probe_count_v) per_step += c ? 1 : 0;
                launches += uint64_t(chunk) * per_step;
                if (check_finite)
                    for (uint32_t c : unit_counts) launches += c ? 1 : 0;
            } else {
                record_chunk(half);
            }
            check(cudaGetLastError(), "chunk launch");
            if (check_finite) {
                check(cudaEventRecord(marked[half], stream), "finite marks");
                marks_pending[half] = true;
                marks_chunk[half] = chunks_run;
            }
        }
        for (auto &kv : entries) {
            Entry &e = kv.second;
            e.step += e.desc.steps;
        }
        stage ^= 1;
        ++chunks_run;
        return stepping;
    }

    void wait(uint32_t timeout_ms) {
        const cudaError_t q = poll_stream(stream, timeout_ms);
        if (q == cudaErrorNotReady) throw Error(DP_ERR_TIMEOUT, "the batch did not finish in time");
        check(q, "stream");
        collect_marks(-1);
        int32_t code = 0;
        check(cudaMemcpy(&code, error, sizeof(code), cudaMemcpyDeviceToHost), "error flag");
        if (code) {
            check(cudaMemset(error, 0, sizeof(int32_t)), "error flag");
            throw Error(DP_ERR_TIMEOUT, "a batch step gave up waiting for its plane loads");
        }
    }
};

namespace {

constexpr uint32_t kTimeoutMs = 600000;

// Bytes a scene needs in the arena.
struct Layout {
    uint32_t pitch, material_pitch;
    uint64_t cells;
    size_t fields, intensity, material, coeff, gains, absorber, weights, probes, total;
};

// Probe series longer than this many values (4 TiB) fit no arena; the
// layout of such a scene reports SIZE_MAX bytes instead of a wrapped product.
constexpr uint64_t kMaxProbeValues = uint64_t(1) << 40;

Layout layout_of(const Scene &s, uint32_t order, uint32_t probe_count, uint64_t steps) {
    Layout l{};
    const uint64_t probe_values = uint64_t(probe_count) * 2;
    if (probe_values && steps > kMaxProbeValues / probe_values) {
        l.total = SIZE_MAX;
        return l;
    }
    uint32_t n[3];
    stored_extent(s.grid.n, order, n);
    l.pitch = (n[0] + 3) / 4 * 4;
    l.material_pitch = (n[0] + 15) / 16 * 16;
    l.cells = uint64_t(l.pitch) * n[1] * n[2];
    const size_t span = size_t(n[0]) + n[1] + n[2];
    l.fields = round_up(3 * l.cells * sizeof(float), kAlign);
    l.intensity = round_up(l.cells * sizeof(float), kAlign);
    l.material = round_up(size_t(l.material_pitch) * n[1] * n[2], kAlign);
    l.coeff = round_up(256 * sizeof(float4), kAlign);
    l.gains = round_up(span * sizeof(float), kAlign);
    l.absorber = round_up(2 * span * sizeof(float), kAlign);
    l.weights = round_up(std::max<size_t>(1, s.weights.size()) * sizeof(float), kAlign);
    l.probes = round_up(std::max<size_t>(1, size_t(probe_count) * steps * 2) * sizeof(float), kAlign);
    l.total = 4 * l.fields + l.intensity + l.material + l.coeff + 2 * l.gains + l.absorber + l.weights + l.probes;
    return l;
}

void make_units(Entry &e, uint32_t planes) {
    const uint32_t *n = e.n;
    const uint32_t tx = 32 * e.variant.cx, ty = e.variant.tile_y;
    const uint32_t tiles_x = (n[0] + tx - 1) / tx, tiles_y = (n[1] + ty - 1) / ty;
    // Units of `planes` planes (at least 8): enough to amortize a unit's
    // start-up (one extra H plane, ring fill), few enough to spread a scene.
    const uint32_t target = std::max<uint32_t>(8, std::min<uint32_t>(planes, n[2]));
    const uint32_t chunks = (n[2] + target - 1) / target;
    const uint32_t depth = (n[2] + chunks - 1) / chunks; // equal chunks, none left short
    e.units.clear();
    for (uint32_t z0 = 0; z0 < n[2]; z0 += depth)
        for (uint32_t ty_i = 0; ty_i < tiles_y; ++ty_i)
            for (uint32_t tx_i = 0; tx_i < tiles_x; ++tx_i)
                e.units.push_back(BatchUnit{e.slot, tx_i * tx, ty_i * ty, z0, std::min(z0 + depth, n[2])});
}

} // namespace

extern "C" {

dp_status dp_batch_create(const dp_batch_options *opts, dp_batch **out) {
    return guarded([&] {
        if (!opts || !out) throw Error(DP_ERR_INVALID, "null argument");
        *out = nullptr;
        auto b = std::make_unique<dp_batch>();
        b->device = opts->device;
        b->chunk = opts->chunk_steps ? opts->chunk_steps : 50;
        b->capacity = opts->max_scenes ? opts->max_scenes : 256;
        b->graphs = opts->use_graphs != 0;
        if (opts->cells_per_lane != 0 && opts->cells_per_lane != 1 && opts->cells_per_lane != 2 &&
            opts->cells_per_lane != 4)
            throw Error(DP_ERR_INVALID, "cells_per_lane must be 0, 1, 2 or 4");
        b->cells_per_lane = opts->cells_per_lane;
        if (opts->axis_order > 6) throw Error(DP_ERR_INVALID, "axis_order must be 0 (per scene) or 1-6");
        b->axis_order = opts->axis_order;
        b->unit_planes = opts->unit_planes ? opts->unit_planes : 24;
        b->unit_planes_set = opts->unit_planes != 0;
        if (opts->arena_bytes == 0) throw Error(DP_ERR_INVALID, "arena_bytes must be positive");
        b->bind();
        check(cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device), "attribute");
        check(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking), "stream");
        configure_batch_kernels();
        check(cudaMalloc(&b->arena_base, opts->arena_bytes), "arena");
        b->arena.reset(opts->arena_bytes);
        b->slot_used.assign(b->capacity, 0);
        check(cudaMalloc(&b->scenes, size_t(b->capacity) * sizeof(BatchScene)), "descriptors");
        check(cudaMemset(b->scenes, 0, size_t(b->capacity) * sizeof(BatchScene)), "descriptors");
        check(cudaMalloc(&b->injections, 2 * b->injection_span() * sizeof(DeviceInjection)), "injections");
        check(cudaMalloc(&b->counts, 2 * b->count_span() * sizeof(uint32_t)), "counts");
        check(cudaMemset(b->counts, 0, 2 * b->count_span() * sizeof(uint32_t)), "counts");
        check(cudaMalloc(&b->error, sizeof(int32_t)), "error");
        check(cudaMemset(b->error, 0, sizeof(int32_t)), "error");
        for (int k = 0; k < 2; ++k) {
            check(cudaMallocHost(&b->h_scenes[k], size_t(b->capacity) * sizeof(BatchScene)), "staging");
            std::memset(b->h_scenes[k], 0, size_t(b->capacity) * sizeof(BatchScene));
            check(cudaMallocHost(&b->h_injections[k], b->injection_span() * sizeof(DeviceInjection)), "staging");
            check(cudaMallocHost(&b->h_counts[k], b->count_span() * sizeof(uint32_t)), "staging");
            check(cudaEventCreateWithFlags(&b->staged[k], cudaEventDisableTiming), "event");
            check(cudaEventRecord(b->staged[k], b->stream), "event");
            check(cudaMallocHost(&b->h_marks[k], size_t(b->capacity) * sizeof(int32_t)), "staging");
            std::memset(b->h_marks[k], 0, size_t(b->capacity) * sizeof(int32_t));
            check(cudaEventCreateWithFlags(&b->marked[k], cudaEventDisableTiming), "event");
        }
        b->check_finite = opts->skip_finite_check == 0;
        check(cudaMalloc(&b->marks, size_t(b->capacity) * sizeof(int32_t)), "finite marks");
        check(cudaMemset(b->marks, 0, size_t(b->capacity) * sizeof(int32_t)), "finite marks");
        *out = b.release();
        return DP_OK;
    });
}

void dp_batch_destroy(dp_batch *batch) { delete batch; }

dp_status dp_batch_add(dp_batch *b, const dp_scene *scene, uint64_t steps, int32_t accumulate_intensity,
                       const uint32_t *probes, uint32_t probe_count, uint64_t *id) {
    return guarded([&] {
        if (!b || !scene || !id || (probe_count && !probes)) throw Error(DP_ERR_INVALID, "null argument");
        const Scene &s = scene_of(scene);
        if (!tensor_maps_available()) throw Error(DP_ERR_UNSUPPORTED, "the CUDA driver offers no tensor-map encoder");
        if (s.injection_slots() > size_t(kBatchInjections))
            throw Error(DP_ERR_UNSUPPORTED, "a batch scene carries at most 8 injection slots (2 per source, 8 for a "
                                            "total-field box)");
        if (s.index_bytes != 1) throw Error(DP_ERR_UNSUPPORTED, "a batch scene carries at most 256 materials");
        uint32_t slot = 0;
        while (slot < b->capacity && b->slot_used[slot]) ++slot;
        if (slot == b->capacity) throw Error(DP_ERR_BUSY, "every scene slot of the batch is in use");
        const uint32_t order = order_for(s, b->axis_order, b->cells_per_lane);
        uint32_t n[3];
        stored_extent(s.grid.n, order, n);
        const Layout l = layout_of(s, order, probe_count, steps);
        if (l.total == SIZE_MAX) throw Error(DP_ERR_OOM, "the probe series of this many steps fit no arena");
        size_t offset = 0;
        for (uint32_t k = 0; k < probe_count; ++k) {
            const uint32_t *c = probes + 3 * k;
            if (c[0] >= s.grid.n[0] || c[1] >= s.grid.n[1] || c[2] >= s.grid.n[2])
                throw Error(DP_ERR_RANGE, "probe outside the grid");
        }
        if (!b->arena.allocate(l.total, offset)) throw Error(DP_ERR_OOM, "the batch arena cannot hold this scene now");
        // The block goes back to the arena if admission fails past this point.
        struct Hold {
            Arena &arena;
            size_t offset, bytes;
            bool kept = false;
            ~Hold() {
                if (!kept) arena.release(offset, bytes);
            }
        } hold{b->arena, offset, l.total};
        b->bind();
        Entry e;
        e.id = b->next_id++;
        e.scene = s;
        e.lines = IncidentLines<float>(s);
        e.slot = slot;
        e.order = order;
        for (int a = 0; a < 3; ++a) e.n[a] = n[a];
        e.variant = variant_in(n, order, b->cells_per_lane);
        TunedPlan tuned{};
        if (b->cells_per_lane == 0 && stored_axis(order, 0) == 0 && tuned_plan(n, b->sm_count, tuned) &&
            tuned.tile_y == 8)
            e.variant = variant_for(n[0], tuned.cx); // the tile width tuned for this shape
        e.pitch = l.pitch;
        e.material_pitch = l.material_pitch;
        e.cells_padded = l.cells;
        e.offset = offset;
        e.bytes = l.total;
        e.target = steps;
        e.accumulate = accumulate_intensity != 0;
        unsigned char *p = b->arena_base + offset;
        auto take = [&](size_t bytes) {
            unsigned char *q = p;
            p += bytes;
            return q;
        };
        BatchScene &d = e.desc;
        std::memset(&d, 0, sizeof(d));
        for (int k = 0; k < 2; ++k) {
            d.e[k] = reinterpret_cast<float *>(take(l.fields));
            d.h[k] = reinterpret_cast<float *>(take(l.fields));
        }
        float *intensity = reinterpret_cast<float *>(take(l.intensity));
        uint8_t *material = take(l.material);
        float4 *coeff = reinterpret_cast<float4 *>(take(l.coeff));
        float *mgain = reinterpret_cast<float *>(take(l.gains));
        float *egain = reinterpret_cast<float *>(take(l.gains));
        float *absorber = reinterpret_cast<float *>(take(l.absorber));
        float *weights = reinterpret_cast<float *>(take(l.weights));
        e.probes = reinterpret_cast<float *>(take(l.probes));
        // Zeroed fields; tables uploaded; the index padded row by row.
        cudaStream_t st = b->stream;
        check(cudaMemsetAsync(b->arena_base + offset, 0, 4 * l.fields + l.intensity, st), "zero fields");
        check(cudaMemsetAsync(b->marks + slot, 0, sizeof(int32_t), st), "finite mark");
        e.joined = b->chunks_run;
        if (order == 0) {
            rasterize_on_device(s, material, l.material_pitch, st);
        } else {
            // Rasterized in the scene's own order, then laid out in the
            // stored one.
            const uint64_t scene_cells = uint64_t(s.grid.n[0]) * s.grid.n[1] * s.grid.n[2];
            uint8_t *own = nullptr;
            check(cudaMallocAsync(reinterpret_cast<void **>(&own), std::max<uint64_t>(1, scene_cells), st), "raster");
            rasterize_on_device(s, own, s.grid.n[0], st);
            const uint64_t total = uint64_t(l.material_pitch) * n[1] * n[2];
            index_to_stored<<<unsigned((total + 255) / 256), 256, 0, st>>>(own, s.grid.n[0], s.grid.n[1], material,
                                                                           l.material_pitch, n[0], n[1], total,
                                                                           axes_of(order));
            check(cudaGetLastError(), "index layout");
            check(cudaFreeAsync(own, st), "raster");
        }
        std::vector<float4> table(256, make_float4(0.0f, 0.0f, 0.0f, 0.0f));
        for (size_t m = 0; m < s.coefficients.size(); ++m)
            table[m] = make_float4(s.coefficients[m].electric_gain, s.coefficients[m].electric_loss,
                                   s.coefficients[m].magnetic_gain, s.coefficients[m].magnetic_loss);
        check(cudaMemcpyAsync(coeff, table.data(), table.size() * sizeof(float4), cudaMemcpyHostToDevice, st), "coeff");
        // The per-axis tables (x | y | z sections) in the stored order.
        auto stored_axes = [&](const float *from, std::vector<float> &to) {
            for (int i = 0; i < 3; ++i) {
                const int a = kBatchAxisOrders[order][i];
                to.insert(to.end(), from + s.axis_offset(a), from + s.axis_offset(a) + s.grid.n[a]);
            }
        };
        const size_t span = size_t(s.grid.n[0]) + s.grid.n[1] + s.grid.n[2];
        std::vector<float> mg, eg, ab;
        stored_axes(s.magnetic_gains.data(), mg);
        stored_axes(s.electric_gains.data(), eg);
        if (reverses_curls(order))
            for (std::vector<float> *g : {&mg, &eg})
                for (float &v : *g) v = -v;
        stored_axes(s.absorber.data(), ab);         // integer samples
        stored_axes(s.absorber.data() + span, ab);  // half-cell samples
        check(cudaMemcpyAsync(mgain, mg.data(), mg.size() * 4, cudaMemcpyHostToDevice, st), "gains");
        check(cudaMemcpyAsync(egain, eg.data(), eg.size() * 4, cudaMemcpyHostToDevice, st), "gains");
        check(cudaMemcpyAsync(absorber, ab.data(), ab.size() * 4, cudaMemcpyHostToDevice, st), "absorber");
        if (!s.weights.empty())
            check(cudaMemcpyAsync(weights, s.weights.data(), s.weights.size() * 4, cudaMemcpyHostToDevice, st), "weights");
        // No wait: copies from pageable memory return once staged, and every
        // later use of these buffers is ordered behind them on the stream.
        for (int a = 0; a < 3; ++a) d.s.n[a] = n[a];
        d.s.pitch = l.pitch;
        d.s.cells = l.cells;
        d.s.material = nullptr; // the fused step reads the index through its tensor map
        d.s.coeff = coeff;
        d.s.mgain = mgain;
        d.s.egain = egain;
        d.s.absorber = absorber;
        d.s.weights = weights;
        d.intensity = e.accumulate ? intensity : nullptr;
        d.scene_z = stored_axis(order, 2);
        try {
            batch_scene_maps(d, e.variant.cx, e.variant.tile_y, material, l.material_pitch);
        } catch (const std::exception &ex) {
            throw Error(DP_ERR_CUDA, ex.what());
        }
        for (uint32_t k = 0; k < probe_count; ++k) {
            const uint32_t *c = probes + 3 * k;
            const int *axes = kBatchAxisOrders[order];
            e.probe_cells.push_back(uint32_t((uint64_t(c[axes[2]]) * n[1] + c[axes[1]]) * l.pitch + c[axes[0]]));
        }
        hold.kept = true;
        b->slot_used[slot] = 1;
        *id = e.id;
        b->entries.emplace(e.id, std::move(e));
        b->dirty = true;
        return DP_OK;
    });
}

dp_status dp_batch_remove(dp_batch *b, uint64_t id) {
    return guarded([&] {
        if (!b) throw Error(DP_ERR_INVALID, "null handle");
        auto it = b->entries.find(id);
        if (it == b->entries.end()) throw Error(DP_ERR_RANGE, "no such scene in the batch");
        b->bind();
        b->wait(kTimeoutMs); // the arena block may still be read by the last chunk
        b->arena.release(it->second.offset, it->second.bytes);
        b->slot_used[it->second.slot] = 0;
        // Clear the slot's staged descriptor so a stale copy never runs.
        for (int k = 0; k < 2; ++k) std::memset(&b->h_scenes[k][it->second.slot], 0, sizeof(BatchScene));
        b->entries.erase(it);
        b->dirty = true;
        return DP_OK;
    });
}

dp_status dp_batch_advance_chunk(dp_batch *b, uint32_t *stepping) {
    return guarded([&] {
        if (!b) throw Error(DP_ERR_INVALID, "null handle");
        b->bind();
        const uint32_t n = b->run_chunk();
        if (stepping) *stepping = n;
        return DP_OK;
    });
}

dp_status dp_batch_wait(dp_batch *b, uint32_t timeout_ms) {
    return guarded([&] {
        if (!b) throw Error(DP_ERR_INVALID, "null handle");
        b->bind();
        b->wait(timeout_ms);
        return DP_OK;
    });
}

dp_status dp_batch_status(dp_batch *b, uint64_t id, uint64_t *step, uint64_t *target) {
    return guarded([&] {
        if (!b || !step || !target) throw Error(DP_ERR_INVALID, "null argument");
        auto it = b->entries.find(id);
        if (it == b->entries.end()) throw Error(DP_ERR_RANGE, "no such scene in the batch");
        *step = it->second.step;
        *target = it->second.target;
        return DP_OK;
    });
}

dp_status dp_batch_fault(dp_batch *b, uint64_t id, dp_status *fault, uint64_t *at_step) {
    return guarded([&] {
        if (!b || !fault) throw Error(DP_ERR_INVALID, "null argument");
        auto it = b->entries.find(id);
        if (it == b->entries.end()) throw Error(DP_ERR_RANGE, "no such scene in the batch");
        b->bind();
        b->collect_marks(-2); // the marks of chunks that have finished; no wait
        *fault = it->second.fault;
        if (at_step) *at_step = it->second.fault == DP_OK ? 0 : it->second.step;
        return DP_OK;
    });
}

dp_status dp_batch_read_field(dp_batch *b, uint64_t id, uint32_t field, float *host, size_t count) {
    return guarded([&] {
        if (!b || !host) throw Error(DP_ERR_INVALID, "null argument");
        auto it = b->entries.find(id);
        if (it == b->entries.end()) throw Error(DP_ERR_RANGE, "no such scene in the batch");
        const Entry &e = it->second;
        const uint32_t *n = e.scene.grid.n;
        const uint64_t cells = uint64_t(n[0]) * n[1] * n[2];
        const int components = field == DP_FIELD_INTENSITY ? 1 : 3;
        if (count != components * cells) throw Error(DP_ERR_RANGE, "element count does not match the field");
        if (field == DP_FIELD_INTENSITY && !e.desc.intensity) throw Error(DP_ERR_INVALID, "intensity is not accumulated");
        b->bind();
        b->wait(kTimeoutMs);
        const uint32_t current = uint32_t(e.step & 1u);
        const float *src = field == DP_FIELD_ELECTRIC ? e.desc.e[current]
                           : field == DP_FIELD_MAGNETIC ? e.desc.h[current] : e.desc.intensity;
        if (field > DP_FIELD_INTENSITY) throw Error(DP_ERR_INVALID, "unknown field");
        if (e.order != 0) {
            // Gathered into the scene's own order on the device first.
            float *dense = nullptr;
            const uint64_t total = uint64_t(components) * cells;
            check(cudaMallocAsync(reinterpret_cast<void **>(&dense), std::max<uint64_t>(1, total) * sizeof(float),
                                  b->stream),
                  "readback");
            Axes comp{{0, 0, 0}};
            if (components == 3)
                for (uint32_t c = 0; c < 3; ++c) comp.a[c] = stored_axis(e.order, c);
            field_from_stored<<<unsigned((total + 255) / 256), 256, 0, b->stream>>>(
                src, e.cells_padded, e.pitch, e.n[1], axes_of(e.order), comp, n[0], n[1], cells, total, dense);
            check(cudaGetLastError(), "readback layout");
            check(cudaMemcpyAsync(host, dense, total * sizeof(float), cudaMemcpyDeviceToHost, b->stream), "readback");
            check(cudaFreeAsync(dense, b->stream), "readback");
        } else {
            try {
                copy_fields_out(host, src, n, e.pitch, e.cells_padded, components, b->stream);
            } catch (const std::runtime_error &ex) {
                throw Error(DP_ERR_CUDA, ex.what());
            }
        }
        b->wait(kTimeoutMs);
        return DP_OK;
    });
}

dp_status dp_batch_read_probes(dp_batch *b, uint64_t id, float *host, size_t count) {
    return guarded([&] {
        if (!b || !host) throw Error(DP_ERR_INVALID, "null argument");
        auto it = b->entries.find(id);
        if (it == b->entries.end()) throw Error(DP_ERR_RANGE, "no such scene in the batch");
        const Entry &e = it->second;
        const size_t n = size_t(e.step) * e.probe_cells.size() * 2;
        if (count > n) throw Error(DP_ERR_RANGE, "more probe values than steps taken");
        b->bind();
        b->wait(kTimeoutMs);
        if (count) check(cudaMemcpy(host, e.probes, count * sizeof(float), cudaMemcpyDeviceToHost), "probes");
        return DP_OK;
    });
}

dp_status dp_batch_memory(const dp_batch *b, uint64_t *used, uint64_t *capacity) {
    return guarded([&] {
        if (!b || !used || !capacity) throw Error(DP_ERR_INVALID, "null argument");
        *used = b->arena.used();
        *capacity = b->arena.capacity();
        return DP_OK;
    });
}

uint64_t dp_scene_batch_bytes(const dp_scene *scene, uint32_t probe_count, uint64_t steps) {
    if (!scene) return 0;
    // The most any axis order the batch may pick takes (rows are padded
    // along the stored x, so the orders differ by a little).
    const Scene &s = scene_of(scene);
    size_t most = 0;
    for (uint32_t order = 0; order < (permutable(s) ? 6u : 1u); ++order)
        most = std::max(most, layout_of(s, order, probe_count, steps).total);
    return most;
}

uint64_t dp_batch_launch_count(const dp_batch *b) { return b ? b->launches : 0; }

dp_status dp_batch_layout(dp_batch *b, uint64_t id, uint32_t *axis_order, uint32_t *tile_width) {
    return guarded([&] {
        if (!b || !axis_order || !tile_width) throw Error(DP_ERR_INVALID, "null argument");
        auto it = b->entries.find(id);
        if (it == b->entries.end()) throw Error(DP_ERR_RANGE, "no such scene in the batch");
        *axis_order = it->second.order;
        *tile_width = 32 * it->second.variant.cx;
        return DP_OK;
    });
}

} // extern "C"
