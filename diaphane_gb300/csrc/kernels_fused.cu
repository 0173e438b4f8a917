// Fused z-streaming step kernel (placeholder until the TMA kernel lands).
#include "device.cuh"

namespace diaphane {

bool fused_supported(const uint32_t n[3]) {
    (void)n;
    return false;
}

FusedPlan fused_plan(const uint32_t n[3], uint32_t tile_y, uint32_t z_chunk, int sm_count) {
    (void)n; (void)tile_y; (void)z_chunk; (void)sm_count;
    return FusedPlan{};
}

void launch_fused_step(const DeviceScene &, const FusedPlan &, FieldSet, FieldSet, float *, const InjectionTable &,
                       uint32_t *, cudaStream_t) {}

} // namespace diaphane
