// Host-side scene resolution: grid spacing, time step, gains, material
// coefficients, absorbing profile, rasterized material index and per-step
// source injections.  Everything the reference's Simulation::new computes on
// the CPU before uploading (src/cpu.rs:100-120, src/gpu.rs:190-319), in f32
// with the reference's operation order so device tables match it bit for bit.
#pragma once

#include "../../include/diaphane_gb300.h"

#include <cstdint>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

namespace diaphane {

// Raised where the reference panics; the C ABI turns it into a status.
struct Error : std::runtime_error {
    dp_status status;
    Error(dp_status s, const std::string &m) : std::runtime_error(m), status(s) {}
};

constexpr float kSpeedOfLight = 299792458.0f;
constexpr float kVacuumPermeability = 1.2566371e-6f;
constexpr float kVacuumPermittivity = 8.854188e-12f;
constexpr float kCourantLimit = 0.57735026f;
constexpr float kPi = 3.14159265358979323846f;

// Cell widths of one axis (Spacing, src/grid.rs:149-286).
struct Axis1D {
    std::vector<float> primary; // corner i to corner i+1
    std::vector<float> dual;    // centre i-1 to centre i
    std::vector<float> corners; // primary.size() + 1 offsets from the low wall

    float length() const { return corners.back(); }
    float finest() const;
    float coarsest() const;
    float worst_ratio() const;
    float position(float coordinate) const;   // cell coordinate -> metres from the centre
    float coordinate(float position) const;   // metres from the centre -> cell coordinate
};

Axis1D axis_uniform(uint32_t count, float width);
Axis1D axis_from_widths(std::vector<float> widths);
Axis1D axis_graded(int axis, float length, float base, const dp_refinement *refinements,
                   uint32_t refinement_count, float max_ratio);

struct ResolvedGrid {
    uint32_t n[3];
    float courant;
    float base; // the base (coarse) cell size, metres
    Axis1D axes[3];

    static ResolvedGrid build(const dp_grid_spec &spec);
    void validate() const;
    uint64_t cells() const { return uint64_t(n[0]) * n[1] * n[2]; }
    float reference_cell_size() const;
    float time_step() const;
    float finest() const;
    float coarsest() const;
    void cell_center(const uint32_t coord[3], float out[3]) const;
    void cell_containing(const float position[3], uint32_t out[3]) const;
    bool contains(const float position[3]) const;
};

struct Coeff {
    float electric_gain, electric_loss, magnetic_gain, magnetic_loss;
};

// One injection slot for one step, ready for a kernel.  T is the type the
// drive value is computed in: f32 for the step itself, f64 for the FP64
// instance (positions and weights stay f32 setup values in both).
template <typename T> struct InjectionOf {
    uint32_t origin[3];
    uint32_t extent[3];
    uint32_t component;
    uint32_t magnetic;
    T value;
    int32_t weight_offset; // into Scene::weights, -1 when every cell weighs 1
    float inverse_waist_squared;
    float center[3];
    // A total-field box's side-face correction varies along the travel axis:
    // a cell then adds value (1) times profile[profile_offset + coord -
    // origin] along profile_axis, from the step's profile values; -1: none.
    int32_t profile_offset = -1;
    uint32_t profile_axis = 0;
};
using StepInjection = InjectionOf<float>;

// The time of step `step`'s injections, (step + 1)·dt, as the step computes
// it: an f32 product for the f32 step, exact in f64 for the FP64 instance.
template <typename T> T step_time(uint64_t step, float dt) {
    if constexpr (std::is_same_v<T, float>) return float(step + 1) * dt;
    else return T(step + 1) * T(dt);
}

// The eight corrections of one total-field box for one step, in application
// order (four on E, then four on H), and the side faces' per-cell values.
template <typename T> struct BoxCorrections {
    std::vector<InjectionOf<T>> items;
    std::vector<T> profiles;
};

// The resolved scene: the tables the kernels read.
struct Scene {
    ResolvedGrid grid;
    dp_boundary boundary;
    std::vector<dp_material> materials;
    std::vector<dp_shape> shapes;
    std::vector<dp_source> sources;

    std::vector<float> magnetic_gains; // nx | ny | nz
    std::vector<float> electric_gains; // nx | ny | nz
    std::vector<float> centers;        // nx | ny | nz
    std::vector<float> primary;        // nx | ny | nz
    std::vector<float> dual;           // nx | ny | nz
    std::vector<float> absorber;       // integer x|y|z then half x|y|z
    std::vector<Coeff> coefficients;
    float absorber_peak = 0.0f;
    bool reversible = false;
    float dt = 0.0f;

    // Apodization weights, precomputed once per sheet source: a sheet's box
    // never moves, so its weights never change.  source_weight[s] is the
    // offset of source s's plane, or -1.
    std::vector<float> weights;
    std::vector<int32_t> source_weight;

  private:
    mutable std::vector<uint8_t> index_cache_;
    mutable bool indexed_ = false;

  public:

    static Scene build(const dp_scene_desc &desc);

    // Scene::material_indices (src/scene.rs:181-206) on the host, computed on
    // first use: index_bytes bytes per cell (u8 up to 256 materials, else a
    // little-endian u16).  The simulation paths rasterize on the device
    // instead (raster.cu); this copy serves the table export and checks.
    const std::vector<uint8_t> &material_index() const;
    uint32_t index_bytes = 1;

    // Grid::cell_lookup (src/grid.rs:635-646): world position (coarse cells
    // from the low corner) to fractional cell coordinate, `samples` per axis.
    std::vector<float> cell_lookup(uint32_t samples) const;
    // The sample count the reference's GPU solver uses (src/gpu.rs:225-228).
    uint32_t lookup_samples() const;
    uint32_t axis_offset(int axis) const { return axis == 0 ? 0 : (axis == 1 ? grid.n[0] : grid.n[0] + grid.n[1]); }

    // Source::injections for every source at `time`, two slots per source
    // (a total-field box, whose corrections depend on the history of its
    // incident line, is refused here).
    void injections(float time, std::vector<StepInjection> &out) const { injections_in<float>(time, out); }
    // The same with time and drive in T (float and double are instantiated).
    // `boxes`, indexed by source, supplies the total-field boxes' corrections
    // of this step; their profile offsets are rebased onto `profiles`.
    template <typename T>
    void injections_in(T time, std::vector<InjectionOf<T>> &out, const std::vector<BoxCorrections<T>> *boxes = nullptr,
                       std::vector<T> *profiles = nullptr) const;
    // Injection slots per step: 8 for a total-field box, 2 for any other source.
    size_t injection_slots() const;
    bool has_boxes() const;
    // A box source's total field in cells: E-node index bounds per axis.
    void box_bounds(const dp_source &src, uint32_t lo[3], uint32_t hi[3]) const;
};

// The incident field of every total-field box of a scene: a 1-D Yee line
// along the box's travel axis, stepped with the grid's own gains there so the
// box faces cancel what the 3-D stencil propagates (dispersion included),
// driven by the one-way plane-wave corrections of src/source.rs:334-401 a few
// cells before the box, and ending in a graded absorbing tail.  The lines'
// state is a function of the step count alone: a request for an earlier step
// replays from the last checkpoint (every 256 steps) before it.
template <typename T> class IncidentLines {
  public:
    IncidentLines() = default;
    explicit IncidentLines(const Scene &scene);
    bool empty() const { return lines_.empty(); }
    // Per source (empty for sources that are not boxes): the corrections of
    // step `step`.  Computed once per step; the lines then stand at step + 1.
    const std::vector<BoxCorrections<T>> &at(uint64_t step);
    // Values of the step's profiles in total, over all boxes.
    size_t profile_width() const { return profile_width_; }

  private:
    struct Line {
        size_t source;
        int a, p, h;                // travel, polarization and incident-H axes
        int lo[3], hi[3];           // the box
        int first;                  // cell index (along a) of element 0
        int inject;                 // element of the line's own plane-wave E row
        std::vector<T> e, hf;       // E at element i, H half an element on
        std::vector<float> ge, gm;  // the grid's gains at those cells
        std::vector<float> le, lm;  // the tail's loss
        dp_source src;
        T gain, retard, h_sign;
        float face_e[2], face_h[2]; // gains along a at the box faces: E at lo, hi; H at lo-1, hi
        float side_h[2], side_e[2]; // gains across: H along h at lo_h-1, hi_h; E along p at lo_p, hi_p
        float sigma_e, sigma_h, sigma_ha, sigma_ea;
    };
    void advance(uint64_t step, std::vector<BoxCorrections<T>> *out);
    std::vector<Line> lines_;
    size_t sources_ = 0;
    float dt_ = 0.0f;
    uint64_t state_ = 0;        // the lines hold E at state_·dt
    uint64_t cached_ = ~0ull;
    std::vector<BoxCorrections<T>> cache_;
    std::vector<std::pair<uint64_t, std::vector<std::vector<T>>>> checkpoints_;
    size_t profile_width_ = 0;
};

// Waveform::evaluate in T (float and double are instantiated).
template <typename T> T waveform_in(const dp_waveform &w, T time);
float injection_weight(const StepInjection &inj, const float position[3]);

// Shape::contains, src/scene.rs:60-81: membership of a cell centre.
bool shape_contains(const dp_shape &s, const float p[3]);
// The cells along `axis` a shape can cover (a conservative range, widened by
// two cells against rounding); lo > hi when it covers none.
void shape_cell_range(const ResolvedGrid &g, const dp_shape &s, int axis, uint32_t &lo, uint32_t &hi);

} // namespace diaphane
