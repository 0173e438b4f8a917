// Per-step profile values of total-field boxes (the side faces' incident
// values along the travel axis), staged through pinned host memory into a
// device ring.  Slot k holds one step's values; its host half is rewritten
// only after the copy that last read it has finished, and its device half is
// overwritten by a copy queued behind the launches that read it (one stream).
#pragma once

#include "setup.hpp"

#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

namespace diaphane {

template <typename T> class ProfileRing {
  public:
    ProfileRing() = default;
    ProfileRing(const ProfileRing &) = delete;
    ProfileRing &operator=(const ProfileRing &) = delete;
    ~ProfileRing() { release(); }

    // `width` values per step, `slots` steps in flight.
    void create(size_t width, uint32_t slots) {
        release();
        if (width == 0) return;
        width_ = width;
        slots_ = slots;
        check(cudaMalloc(reinterpret_cast<void **>(&device_), width * slots * sizeof(T)), "profile ring");
        check(cudaMallocHost(reinterpret_cast<void **>(&host_), width * slots * sizeof(T)), "profile staging");
        copied_.assign(slots, nullptr);
        pending_.assign(slots, 0);
        for (auto &e : copied_) check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming), "profile event");
    }

    void release() {
        for (auto &e : copied_)
            if (e) cudaEventDestroy(e);
        copied_.clear();
        pending_.clear();
        if (device_) cudaFree(device_);
        if (host_) cudaFreeHost(host_);
        device_ = nullptr;
        host_ = nullptr;
        width_ = 0;
        slots_ = next_ = 0;
    }

    // Stages one step's values (at most `width`) and queues their copy on
    // `stream`; returns the device address the step's launches read.
    const T *put(const std::vector<T> &values, cudaStream_t stream) {
        if (values.size() > width_) throw Error(DP_ERR_CUDA, "profile values exceed the ring's width");
        const uint32_t k = next_;
        next_ = (next_ + 1) % slots_;
        if (pending_[k]) check(cudaEventSynchronize(copied_[k]), "profile staging");
        T *host = host_ + size_t(k) * width_;
        T *device = device_ + size_t(k) * width_;
        std::memcpy(host, values.data(), values.size() * sizeof(T));
        check(cudaMemcpyAsync(device, host, values.size() * sizeof(T), cudaMemcpyHostToDevice, stream), "profiles");
        check(cudaEventRecord(copied_[k], stream), "profile event");
        pending_[k] = 1;
        return device;
    }

  private:
    static void check(cudaError_t err, const char *what) {
        if (err != cudaSuccess) {
            cudaGetLastError();
            throw Error(err == cudaErrorMemoryAllocation ? DP_ERR_OOM : DP_ERR_CUDA,
                        std::string(what) + ": " + cudaGetErrorString(err));
        }
    }

    T *device_ = nullptr;
    T *host_ = nullptr;
    std::vector<cudaEvent_t> copied_;
    std::vector<char> pending_;
    size_t width_ = 0;
    uint32_t slots_ = 0, next_ = 0;
};

} // namespace diaphane
