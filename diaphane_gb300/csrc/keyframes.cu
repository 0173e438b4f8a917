// C ABI: a keyframe ring kept in device memory (Timeline, src/timeline.rs:76-213).
//
// The reference's timeline snapshots both fields to the host every so often
// and seeks backwards by restoring the newest keyframe at or before the
// target and replaying the remainder.  Here a keyframe is a device-to-device
// copy of the current E and H buffers into a slot of one preallocated block,
// and a restore is the copy back, both ordered on the simulation's stream:
// no host round trip, so a scrub costs the replay and two HBM copies.
// The policy — when a keyframe is due, which one a seek restores, falling
// back to a reset when the window has slid past the target — is the
// reference's (src/timeline.rs:137-212).
#include "sim.hpp"

#include <deque>

namespace {

struct Frame {
    uint64_t step;
    uint32_t slot;
};

} // namespace

struct dp_keyframes {
    dp_sim *sim = nullptr;
    uint64_t interval = 0;
    uint32_t capacity = 0;
    float *store = nullptr;   // capacity slots of (E, H), each 3 × padded cells
    uint64_t slot_floats = 0; // floats per slot
    std::deque<Frame> frames; // oldest first
    std::vector<uint32_t> free_slots;

    ~dp_keyframes() {
        if (sim && sim->stream) {
            cudaSetDevice(sim->device);
            cudaStreamSynchronize(sim->stream);
        }
        cudaFree(store);
    }

    float *slot_ptr(uint32_t slot) const { return store + slot * slot_floats; }

    void snapshot_into(uint32_t slot) {
        const uint64_t n = 3 * sim->padded_cells();
        const FieldSet f = sim->fields();
        check_cuda(cudaMemcpyAsync(slot_ptr(slot), f.e, n * sizeof(float), cudaMemcpyDeviceToDevice, sim->stream),
                   "keyframe");
        check_cuda(cudaMemcpyAsync(slot_ptr(slot) + n, f.h, n * sizeof(float), cudaMemcpyDeviceToDevice, sim->stream),
                   "keyframe");
    }

    // Restore (Steppable::restore): the fields of the frame, its step, and
    // an empty intensity average (it belonged to the abandoned history).
    void restore_from(const Frame &frame) {
        const uint64_t n = 3 * sim->padded_cells();
        sim->clear_intensity();
        const FieldSet f = sim->fields();
        check_cuda(cudaMemcpyAsync(f.e, slot_ptr(frame.slot), n * sizeof(float), cudaMemcpyDeviceToDevice, sim->stream),
                   "restore");
        check_cuda(cudaMemcpyAsync(f.h, slot_ptr(frame.slot) + n, n * sizeof(float), cudaMemcpyDeviceToDevice,
                                   sim->stream),
                   "restore");
        sim->step = frame.step;
        sim->probe_since = frame.step;
    }

    // Timeline::observe, src/timeline.rs:137-154.
    void observe() {
        const uint64_t step = sim->step;
        uint64_t newest = 0;
        if (!frames.empty()) {
            const uint64_t last = frames.back().step;
            if (step <= last) return; // replaying covered ground after a backward seek
            newest = last / interval;
        }
        if (step / interval <= newest) return;
        if (frames.size() == capacity) {
            free_slots.push_back(frames.front().slot);
            frames.pop_front();
        }
        const uint32_t slot = free_slots.back();
        free_slots.pop_back();
        snapshot_into(slot);
        frames.push_back(Frame{step, slot});
    }

    // Timeline::seek, src/timeline.rs:180-212.
    dp_seek seek(uint64_t target) {
        const uint64_t current = sim->step;
        if (target == current) return dp_seek{DP_SEEK_UNCHANGED, 0, 0};
        if (target > current) {
            sim->forward(target - current);
            return dp_seek{DP_SEEK_FORWARD, target - current, 0};
        }
        for (auto it = frames.rbegin(); it != frames.rend(); ++it) {
            if (it->step <= target) {
                restore_from(*it);
                sim->forward(target - it->step);
                return dp_seek{DP_SEEK_KEYFRAME, target - it->step, it->step};
            }
        }
        sim->reset_fields();
        sim->forward(target);
        return dp_seek{DP_SEEK_START, target, 0};
    }

    void clear() {
        for (const Frame &f : frames) free_slots.push_back(f.slot);
        frames.clear();
    }
};

extern "C" {

dp_status dp_keyframes_create(dp_sim *sim, uint64_t interval, uint32_t capacity, dp_keyframes **out) {
    return guarded([&] {
        if (!sim || !out) throw Error(DP_ERR_INVALID, "null argument");
        *out = nullptr;
        if (interval == 0) throw Error(DP_ERR_INVALID, "keyframe interval must be positive");
        if (capacity == 0) throw Error(DP_ERR_INVALID, "a timeline needs room for at least one keyframe");
        auto k = std::make_unique<dp_keyframes>();
        k->sim = sim;
        k->interval = interval;
        k->capacity = capacity;
        k->slot_floats = 6 * sim->padded_cells();
        if (capacity > SIZE_MAX / sizeof(float) / k->slot_floats)
            throw Error(DP_ERR_OOM, "a keyframe store larger than the address space");
        sim->bind();
        check_cuda(cudaMalloc(&k->store, size_t(capacity) * k->slot_floats * sizeof(float)), "keyframe store");
        for (uint32_t s = capacity; s-- > 0;) k->free_slots.push_back(s);
        *out = k.release();
        return DP_OK;
    });
}

void dp_keyframes_destroy(dp_keyframes *k) { delete k; }

dp_status dp_keyframes_observe(dp_keyframes *k) {
    return guarded([&] {
        if (!k) throw Error(DP_ERR_INVALID, "null handle");
        k->sim->bind();
        k->observe();
        return DP_OK;
    });
}

dp_status dp_keyframes_seek(dp_keyframes *k, uint64_t target, dp_seek *out) {
    return guarded([&] {
        if (!k) throw Error(DP_ERR_INVALID, "null handle");
        k->sim->bind();
        const dp_seek r = k->seek(target);
        if (out) *out = r;
        return DP_OK;
    });
}

dp_status dp_keyframes_clear(dp_keyframes *k) {
    return guarded([&] {
        if (!k) throw Error(DP_ERR_INVALID, "null handle");
        k->clear();
        return DP_OK;
    });
}

uint32_t dp_keyframes_count(const dp_keyframes *k) { return k ? uint32_t(k->frames.size()) : 0; }

dp_status dp_keyframes_earliest(const dp_keyframes *k, uint64_t *step) {
    return guarded([&] {
        if (!k || !step) throw Error(DP_ERR_INVALID, "null argument");
        if (k->frames.empty()) throw Error(DP_ERR_RANGE, "no keyframes yet");
        *step = k->frames.front().step;
        return DP_OK;
    });
}

uint64_t dp_keyframes_bytes(const dp_keyframes *k) {
    return k ? uint64_t(k->frames.size()) * 24 * k->sim->scene.grid.cells() : 0;
}

} // extern "C"
