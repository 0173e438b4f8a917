// ORACLE — test infrastructure only.
//
// A CPU restatement of the reference solver (kvark/diaphane, Rust) used as the
// checker for the CUDA path.  Only the tests, __graft_entry__.smoke() and
// bench.py's CPU-baseline legs load it; nothing in the product links it.
//
// It follows the reference line by line, in the same arithmetic order, so that
// the f32 instance reproduces the Rust f32 results bit for bit:
//   * compiled with -ffp-contract=off (Rust never contracts a*b+c into an FMA);
//   * Rust's f32::{exp, sin, cos, asin, ln, powf} go to the platform libm, and
//     so do expf/sinf/cosf/asinf/logf/powf here;
//   * a+b+c in Rust is (a+b)+c, and that grouping is kept everywhere.
// The FP64 instance runs the same stepping in double (gains, losses and
// injection values promoted from their f32 setup values; waveforms evaluated
// in double) and is the "FP64 CPU run of the same scene".
//
// Parity pinning: the reference ships no golden vectors (its tests are
// analytic and differential), and its Rust toolchain is absent here, so this
// restatement is pinned by re-running the reference's own analytic acceptance
// tests and unit known-answer tests against it (tests/test_oracle_*.py).
//
// Sections and the reference code each follows:
//   Spacing / grade / Grid ........ src/grid.rs:165-286, 405-613, 695-745, 791-888
//   numerical_phase_velocity ...... src/grid.rs:966-1012
//   Material coefficients ......... src/material.rs:77-122
//   AbsorbingProfile .............. src/boundary.rs:100-196
//   Waveform / Source / Injection . src/source.rs:74-115, 280-403, 441-455
//   Shape / material_indices ...... src/scene.rs:60-81, 181-206
//   Simulation .................... src/cpu.rs:100-713

#include "../include/diaphane_gb300.h"

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <memory>
#include <string>
#include <vector>

#ifdef _OPENMP
#include <omp.h>
#endif

namespace oracle {

constexpr float SPEED_OF_LIGHT = 299792458.0f;              // src/grid.rs:42
constexpr float VACUUM_PERMEABILITY = 1.2566371e-6f;        // src/grid.rs:44
constexpr float VACUUM_PERMITTIVITY = 8.854188e-12f;        // src/grid.rs:46
constexpr float COURANT_LIMIT = 0.57735026f;                // src/grid.rs:411
constexpr float PI_F = 3.14159265358979323846f;             // f32::consts::PI

static thread_local std::string last_error;

struct Panic {
    std::string message;
};

[[noreturn]] static void panic(const std::string &message) { throw Panic{message}; }

// Rust `f32 as u32` saturates; C casts of out-of-range floats are undefined.
static uint32_t f32_to_u32(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 4294967296.0f) return UINT32_MAX;
    return static_cast<uint32_t>(v);
}
static size_t f32_to_usize(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 1.8446744e19f) return SIZE_MAX;
    return static_cast<size_t>(v);
}

// ---------------------------------------------------------------------------
// Spacing — src/grid.rs:149-286
// ---------------------------------------------------------------------------
struct Spacing {
    std::vector<float> primary, dual, corners;

    static Spacing assemble(std::vector<float> primary, std::vector<float> corners) {
        if (primary.size() < 2) panic("an axis needs at least 2 cells");
        for (float w : primary)
            if (!(w > 0.0f && std::isfinite(w))) panic("cell widths must be positive and finite");
        Spacing s;
        s.dual.resize(primary.size());
        for (size_t i = 0; i < primary.size(); ++i) {
            size_t prev = i == 0 ? 0 : i - 1;
            s.dual[i] = 0.5f * (primary[prev] + primary[i]);
        }
        s.primary = std::move(primary);
        s.corners = std::move(corners);
        return s;
    }

    // src/grid.rs:167-178: corners multiplied in f64, not accumulated.
    static Spacing uniform(uint32_t count, float width) {
        if (count < 2) panic("an axis needs at least 2 cells");
        std::vector<float> corners(count + 1);
        for (uint32_t i = 0; i <= count; ++i)
            corners[i] = static_cast<float>(static_cast<double>(i) * static_cast<double>(width));
        return assemble(std::vector<float>(count, width), std::move(corners));
    }

    // src/grid.rs:181-190: corners summed in f64.
    static Spacing from_widths(std::vector<float> primary) {
        std::vector<float> corners;
        corners.reserve(primary.size() + 1);
        double offset = 0.0;
        corners.push_back(0.0f);
        for (float w : primary) {
            offset += static_cast<double>(w);
            corners.push_back(static_cast<float>(offset));
        }
        return assemble(std::move(primary), std::move(corners));
    }

    uint32_t count() const { return static_cast<uint32_t>(primary.size()); }
    float length() const { return corners.back(); }
    float finest() const {
        float m = std::numeric_limits<float>::infinity();
        for (float w : primary) m = std::fmin(m, w);
        return m;
    }
    float coarsest() const {
        float m = -std::numeric_limits<float>::infinity();
        for (float w : primary) m = std::fmax(m, w);
        return m;
    }
    float worst_ratio() const {
        float m = 1.0f;
        for (size_t i = 0; i + 1 < primary.size(); ++i)
            m = std::fmax(m, std::fmax(primary[i + 1] / primary[i], primary[i] / primary[i + 1]));
        return m;
    }
    float offset_of(float coordinate) const {
        size_t last = primary.size() - 1;
        size_t index = std::min(f32_to_usize(std::fmax(std::floor(coordinate), 0.0f)), last);
        return corners[index] + (coordinate - static_cast<float>(index)) * primary[index];
    }
    float position(float coordinate) const { return offset_of(coordinate) - 0.5f * length(); }
    float coordinate(float position) const {
        float offset = position + 0.5f * length();
        // partition_point(|c| c <= offset): first corner strictly past offset.
        size_t pp = static_cast<size_t>(std::upper_bound(corners.begin(), corners.end(), offset) -
                                        corners.begin());
        size_t index = pp == 0 ? 0 : pp - 1;
        index = std::min(index, primary.size() - 1);
        return static_cast<float>(index) + (offset - corners[index]) / primary[index];
    }
};

// grade() — src/grid.rs:791-888.
static Spacing grade(size_t axis, float length, float base, const std::vector<dp_refinement> &all,
                     float max_ratio) {
    std::vector<const dp_refinement *> refinements;
    for (const auto &r : all)
        if (r.size[axis] > 0.0f) refinements.push_back(&r);
    if (refinements.empty())
        return Spacing::uniform(f32_to_u32(std::fmax(std::round(length / base), 2.0f)), base);
    float finest = base;
    for (auto *r : refinements) finest = std::fmin(finest, r->cell_size);
    if (!(finest > 0.0f && std::isfinite(finest)))
        panic("refinement cell sizes must be positive and finite");
    size_t samples = f32_to_usize(std::ceil(length / finest * 4.0f));
    samples = std::clamp<size_t>(samples, 64, size_t(1) << 20);
    float step = length / static_cast<float>(samples);

    std::vector<float> target(samples + 1, base);
    for (size_t index = 0; index < target.size(); ++index) {
        float position = static_cast<float>(index) * step - 0.5f * length;
        for (auto *r : refinements) {
            float half = 0.5f * r->size[axis];
            if (std::fabs(position - r->center[axis]) <= half)
                target[index] = std::fmin(target[index], r->cell_size);
        }
    }
    float slope = (max_ratio - 1.0f) * step;
    for (size_t i = 1; i < target.size(); ++i) target[i] = std::fmin(target[i], target[i - 1] + slope);
    for (size_t i = target.size() - 1; i-- > 0;) target[i] = std::fmin(target[i], target[i + 1] + slope);

    std::vector<float> widths;
    float offset = 0.0f;
    while (offset < length) {
        size_t index = std::min(f32_to_usize(offset / step), target.size() - 1);
        widths.push_back(target[index]);
        offset += target[index];
        if (widths.size() > (size_t(1) << 16)) panic("grading ran to too many cells");
    }
    for (size_t i = 1; i < widths.size(); ++i) widths[i] = std::fmin(widths[i], widths[i - 1] * max_ratio);
    for (size_t i = widths.size() - 1; i-- > 0;) widths[i] = std::fmin(widths[i], widths[i + 1] * max_ratio);

    float total = 0.0f;
    for (float w : widths) total += w;
    if (widths.size() > 2) {
        float without = total - widths.back();
        if (std::fabs(length - without) < std::fabs(total - length)) {
            widths.pop_back();
            total = without;
        }
    }
    float scale = length / total;
    for (float &w : widths) w *= scale;
    return Spacing::from_widths(std::move(widths));
}

// ---------------------------------------------------------------------------
// Grid — src/grid.rs:345-774
// ---------------------------------------------------------------------------
struct Grid {
    uint32_t extent[3];
    float courant;
    Spacing spacing[3];

    static Grid build(const dp_grid_spec &spec) {
        float base_cell = spec.cell_size;
        if (!(base_cell > 0.0f && std::isfinite(base_cell))) panic("cell size must be positive and finite");
        if (!(spec.max_ratio > 1.0f && std::isfinite(spec.max_ratio))) panic("the growth cap must exceed 1");
        std::vector<dp_refinement> refinements(spec.refinements, spec.refinements + spec.refinement_count);
        Grid g;
        for (size_t axis = 0; axis < 3; ++axis) {
            if (refinements.empty())
                g.spacing[axis] = Spacing::uniform(spec.extent[axis], base_cell);
            else
                g.spacing[axis] = grade(axis, static_cast<float>(spec.extent[axis]) * base_cell, base_cell,
                                        refinements, spec.max_ratio);
            g.extent[axis] = g.spacing[axis].count();
        }
        g.courant = spec.courant;
        return g;
    }

    void validate() const {
        for (int a = 0; a < 3; ++a)
            if (extent[a] < 2) panic("grid must be at least 2 cells across on every axis");
        if (!(courant > 0.0f && courant <= COURANT_LIMIT)) panic("Courant number is outside (0, limit]");
    }
    size_t total() const { return size_t(extent[0]) * extent[1] * extent[2]; }
    size_t index(size_t x, size_t y, size_t z) const { return (z * extent[1] + y) * extent[0] + x; }
    float finest() const {
        float m = std::numeric_limits<float>::infinity();
        for (int a = 0; a < 3; ++a) m = std::fmin(m, spacing[a].finest());
        return m;
    }
    float coarsest() const {
        float m = -std::numeric_limits<float>::infinity();
        for (int a = 0; a < 3; ++a) m = std::fmax(m, spacing[a].coarsest());
        return m;
    }
    // src/grid.rs:575-584
    float reference_cell_size() const {
        float inverse_squares = -0.0f;
        for (int a = 0; a < 3; ++a) {
            float f = spacing[a].finest();
            inverse_squares = inverse_squares + 1.0f / (f * f);
        }
        return std::sqrt(3.0f / inverse_squares);
    }
    float time_step() const { return courant * reference_cell_size() / SPEED_OF_LIGHT; }
    std::vector<float> gains(const std::vector<float> &widths) const {
        float travel = SPEED_OF_LIGHT * time_step();
        std::vector<float> g(widths.size());
        for (size_t i = 0; i < widths.size(); ++i) g[i] = travel / widths[i];
        return g;
    }
    std::vector<float> magnetic_gains(int axis) const { return gains(spacing[axis].primary); }
    std::vector<float> electric_gains(int axis) const { return gains(spacing[axis].dual); }
    float size(int axis) const { return spacing[axis].length(); }
    std::vector<float> cell_centers(int axis) const {
        std::vector<float> c(extent[axis]);
        for (uint32_t i = 0; i < extent[axis]; ++i) c[i] = spacing[axis].position(static_cast<float>(i) + 0.5f);
        return c;
    }
    void cell_center(const size_t coord[3], float out[3]) const {
        for (int a = 0; a < 3; ++a) out[a] = spacing[a].position(static_cast<float>(coord[a]) + 0.5f);
    }
    void cell_containing(const float position[3], size_t out[3]) const {
        for (int a = 0; a < 3; ++a) {
            float cell = spacing[a].coordinate(position[a]);
            out[a] = std::min(f32_to_usize(std::fmax(std::floor(cell), 0.0f)), size_t(extent[a]) - 1);
        }
    }
    bool contains(const float position[3]) const {
        for (int a = 0; a < 3; ++a)
            if (!(std::fabs(position[a]) <= 0.5f * size(a))) return false;
        return true;
    }
    float frequency_for_resolution(float cells) const { return SPEED_OF_LIGHT / (cells * coarsest()); }
};

// numerical_phase_velocity — src/grid.rs:966-1012 (analysis code, f64).
static float numerical_phase_velocity(float courant_f, float cells_f, const float direction[3]) {
    double courant = courant_f, cells = cells_f;
    double norm = 0.0;
    for (int i = 0; i < 3; ++i) norm += double(direction[i]) * double(direction[i]);
    norm = std::sqrt(norm);
    double unit[3];
    for (int i = 0; i < 3; ++i) unit[i] = double(direction[i]) / norm;
    double s = std::sin(M_PI * courant / cells) / courant;
    double target = s * s;
    auto residual = [&](double k) {
        double sum = 0.0;
        for (int i = 0; i < 3; ++i) {
            double v = std::sin(0.5 * k * unit[i]);
            sum += v * v;
        }
        return sum - target;
    };
    double ideal = 2.0 * M_PI / cells;
    double lo = 0.5 * ideal, hi = 2.0 * ideal;
    for (int i = 0; i < 80; ++i) {
        double mid = 0.5 * (lo + hi);
        if (residual(mid) < 0.0) lo = mid; else hi = mid;
    }
    return static_cast<float>(ideal / (0.5 * (lo + hi)));
}

// ---------------------------------------------------------------------------
// Materials — src/material.rs:100-122
// ---------------------------------------------------------------------------
struct Coefficients {
    float electric_gain, electric_loss, magnetic_gain, magnetic_loss;
};

static Coefficients coefficients(const dp_material &m, const Grid &grid) {
    if (std::isinf(m.conductivity))
        return Coefficients{0.0f, 1.0f, 1.0f / m.relative_permeability, 0.0f};
    float half_step = 0.5f * grid.time_step();
    return Coefficients{
        1.0f / m.relative_permittivity,
        half_step * m.conductivity / (VACUUM_PERMITTIVITY * m.relative_permittivity),
        1.0f / m.relative_permeability,
        half_step * m.magnetic_loss / (VACUUM_PERMEABILITY * m.relative_permeability),
    };
}

// ---------------------------------------------------------------------------
// AbsorbingProfile — src/boundary.rs:100-196
// ---------------------------------------------------------------------------
struct Absorber {
    std::vector<float> integer[3], half[3];

    static Absorber build(const Grid &grid, const dp_boundary &b) {
        Absorber p;
        size_t thickness = b.kind == DP_BOUNDARY_PEC ? 0 : b.thickness;
        float target = b.kind == DP_BOUNDARY_PEC ? 1.0f : b.target_reflection;
        if (thickness == 0) {
            for (int a = 0; a < 3; ++a) {
                p.integer[a].assign(grid.extent[a], 0.0f);
                p.half[a].assign(grid.extent[a], 0.0f);
            }
            return p;
        }
        for (int a = 0; a < 3; ++a)
            if (!(2 * thickness < grid.extent[a])) panic("absorbing layers do not fit in the axis");
        if (!(target > 0.0f && target < 1.0f)) panic("target reflection must lie in (0, 1)");
        const float order = 3.0f;
        float peak = -(order + 1.0f) * std::log(target) * grid.courant / (4.0f * static_cast<float>(thickness));
        float t = static_cast<float>(thickness);
        auto profile = [&](float position, size_t n) {
            float outer = static_cast<float>(n - 1);
            float depth_low = (t - position) / t;
            float depth_high = (t - (outer - position)) / t;
            float depth = std::fmax(depth_low, depth_high);
            depth = depth < 0.0f ? 0.0f : (depth > 1.0f ? 1.0f : depth);
            return peak * std::pow(depth, order);
        };
        for (int a = 0; a < 3; ++a) {
            size_t n = grid.extent[a];
            p.integer[a].resize(n);
            p.half[a].resize(n);
            for (size_t i = 0; i < n; ++i) {
                p.integer[a][i] = profile(static_cast<float>(i), n);
                p.half[a][i] = profile(static_cast<float>(i) + 0.5f, n);
            }
        }
        return p;
    }
    // electric_row / magnetic_row: (varying along x, constant for the row).
    const std::vector<float> &pick(bool electric, int axis, int t) const {
        bool use_half = electric ? (t == axis) : (t != axis);
        return use_half ? half[t] : integer[t];
    }
    float peak() const {
        float m = 0.0f;
        for (int a = 0; a < 3; ++a) {
            for (float v : half[a]) m = std::fmax(m, v);
            for (float v : integer[a]) m = std::fmax(m, v);
        }
        return m;
    }
};

// ---------------------------------------------------------------------------
// Waveforms and sources — src/source.rs:74-455
// ---------------------------------------------------------------------------
template <typename T> struct Math;
template <> struct Math<float> {
    static float exp(float v) { return std::exp(v); }
    static float sin(float v) { return std::sin(v); }
    static float cos(float v) { return std::cos(v); }
    static constexpr float pi = PI_F;
};
template <> struct Math<double> {
    static double exp(double v) { return std::exp(v); }
    static double sin(double v) { return std::sin(v); }
    static double cos(double v) { return std::cos(v); }
    static constexpr double pi = M_PI;
};

template <typename T> static T evaluate(const dp_waveform &w, T time) {
    using M = Math<T>;
    switch (w.kind) {
    case DP_WAVE_RICKER: {
        T arg = M::pi * T(w.frequency) * (time - T(w.delay));
        T arg2 = arg * arg;
        return (T(1) - T(2) * arg2) * M::exp(-arg2);
    }
    case DP_WAVE_GAUSSIAN_PULSE: {
        const T FWHM_TO_SIGMA = T(0.4246609f);
        T sigma = FWHM_TO_SIGMA * T(w.duration_cycles) / T(w.frequency);
        T tau = time - T(w.delay);
        T envelope = M::exp(T(-0.5) * (tau / sigma) * (tau / sigma));
        return envelope * M::sin(T(2) * M::pi * T(w.frequency) * tau);
    }
    default: {
        if (time <= T(0)) return T(0);
        T ramp_duration = T(w.ramp_cycles) / T(w.frequency);
        T envelope = time >= ramp_duration ? T(1) : T(0.5) * (T(1) - M::cos(M::pi * time / ramp_duration));
        return envelope * M::sin(T(2) * M::pi * T(w.frequency) * time);
    }
    }
}

template <typename T> struct Injection {
    size_t origin[3];
    size_t extent[3];
    float center[3];
    float inverse_waist_squared;
    int component;
    bool magnetic;
    T value;

    // src/source.rs:441-455 (apodization stays f32, a geometric setup value).
    float weight(const float position[3]) const {
        if (inverse_waist_squared == 0.0f) return 1.0f;
        float r2 = 0.0f;
        for (int a = 0; a < 3; ++a) {
            if (extent[a] > 1) {
                float offset = position[a] - center[a];
                r2 += offset * offset;
            }
        }
        return std::exp(-r2 * inverse_waist_squared);
    }
};

// Source::injections — src/source.rs:280-403.  The time arithmetic follows
// the reference in T; positions stay f32 as the reference's are.
template <typename T>
static void injections(const dp_source &s, const Grid &grid, T time, Injection<T> out[2]) {
    T value = T(s.amplitude) * evaluate<T>(s.waveform, time);
    for (int i = 0; i < 2; ++i) {
        std::memset(&out[i], 0, sizeof(out[i]));
        out[i].component = int(s.polarization);
    }
    switch (s.shape) {
    case DP_SOURCE_POINT: {
        float position[3];
        for (int a = 0; a < 3; ++a) position[a] = s.at[a] + s.velocity[a] * static_cast<float>(time);
        Injection<T> inj{};
        grid.cell_containing(position, inj.origin);
        inj.extent[0] = inj.extent[1] = inj.extent[2] = 1;
        inj.component = int(s.polarization);
        inj.magnetic = false;
        inj.value = grid.contains(position) ? value : T(0);
        out[0] = inj;
        out[1] = inj;
        out[1].value = T(0);
        return;
    }
    case DP_SOURCE_SHEET: {
        int a = int(s.axis);
        float position[3] = {0.0f, 0.0f, 0.0f};
        position[a] = s.offset;
        size_t cell[3];
        grid.cell_containing(position, cell);
        Injection<T> inj{};
        for (int t = 0; t < 3; ++t) {
            inj.origin[t] = 0;
            inj.extent[t] = grid.extent[t];
        }
        inj.origin[a] = cell[a];
        inj.extent[a] = 1;
        inj.inverse_waist_squared = 1.0f / (s.waist * s.waist);
        inj.component = int(s.polarization);
        inj.magnetic = false;
        inj.value = value;
        out[0] = inj;
        out[1] = inj;
        out[1].value = T(0);
        return;
    }
    default: {
        int travel = int(s.axis);
        float position[3] = {0.0f, 0.0f, 0.0f};
        position[travel] = s.offset;
        size_t cell[3];
        grid.cell_containing(position, cell);
        size_t plane = std::max<size_t>(cell[travel], 1);
        float spacing = grid.spacing[travel].finest();
        float time_step_f = grid.time_step();
        float gain_f = SPEED_OF_LIGHT * time_step_f / spacing;
        T time_step = T(time_step_f);
        T gain = T(gain_f);
        T omega = T(2) * Math<T>::pi * T(s.waveform.frequency);
        T half_k = std::asin(Math<T>::sin(T(0.5) * omega * time_step) / gain);
        T retard = half_k / omega;
        int pol = int(s.polarization);
        int h_axis = 3 - travel - pol;
        T h_sign = ((pol + 1) % 3) == travel ? T(-1) : T(1);
        auto drive = [&](T t) { return T(s.amplitude) * evaluate<T>(s.waveform, t); };
        Injection<T> e{}, h{};
        for (int t = 0; t < 3; ++t) {
            e.extent[t] = h.extent[t] = grid.extent[t];
        }
        e.origin[travel] = plane;
        e.extent[travel] = 1;
        h.origin[travel] = plane - 1;
        h.extent[travel] = 1;
        e.component = pol;
        e.magnetic = false;
        e.value = gain * drive(time - T(0.5) * time_step + retard);
        h.component = h_axis;
        h.magnetic = true;
        h.value = h_sign * gain * drive(time - time_step);
        out[0] = e;
        out[1] = h;
        return;
    }
    }
}

// ---------------------------------------------------------------------------
// Scene rasterization — src/scene.rs:60-81, 181-206
// ---------------------------------------------------------------------------
static bool shape_contains(const dp_shape &s, const float p[3]) {
    switch (s.kind) {
    case DP_SHAPE_BLOCK:
        for (int a = 0; a < 3; ++a)
            if (!(std::fabs(p[a] - s.center[a]) <= 0.5f * s.size[a])) return false;
        return true;
    case DP_SHAPE_SPHERE: {
        float d2 = -0.0f;
        for (int a = 0; a < 3; ++a) {
            float o = p[a] - s.center[a];
            d2 = d2 + o * o;
        }
        return d2 <= s.radius * s.radius;
    }
    default:
        return std::fabs(p[s.axis] - s.offset) <= 0.5f * s.thickness;
    }
}

static std::vector<uint32_t> material_indices(const Grid &grid, const std::vector<dp_shape> &shapes) {
    std::vector<uint32_t> indices(grid.total(), 0);
    if (shapes.empty()) return indices;
    const long nz = grid.extent[2];
#pragma omp parallel for schedule(static)
    for (long z = 0; z < nz; ++z)
        for (size_t y = 0; y < grid.extent[1]; ++y)
            for (size_t x = 0; x < grid.extent[0]; ++x) {
                size_t coord[3] = {x, y, size_t(z)};
                float position[3];
                grid.cell_center(coord, position);
                uint32_t m = 0;
                for (const auto &s : shapes)
                    if (shape_contains(s, position)) m = s.material;
                indices[grid.index(x, y, size_t(z))] = m;
            }
    return indices;
}

// ---------------------------------------------------------------------------
// Total-field box (DP_SOURCE_PLANE_WAVE_BOX).  An extension with no reference
// counterpart: the reference's plane wave (src/source.rs:334-401) spans the
// whole cross-section.  Restated here from the library's specification, not
// from its code: a node of the Yee cell is total when its position lies in
// the box (E_q on lo..hi-1 along q, lo..hi across; H_q the other way round);
// an update reading across the surface is corrected by its coefficient times
// the incident value at the node it read, which leaves E_p and H_h on the two
// faces across the travel axis a and the travel components on the side
// faces, H_a across h and E_a across p.  The incident field is a 1-D Yee line
// along a with the grid's gains there, driven by the plane wave's two
// corrections four cells before the box and ending in a 64-cell graded
// absorbing tail.  Pinned by the one-way test method of tests/validation.rs:
// 375-429 (the field outside the box stays at roundoff).
// ---------------------------------------------------------------------------
template <typename T> struct BoxSource {
    struct Face {
        int component;
        bool magnetic;
        size_t origin[3], extent[3];
        T value;                 // uniform faces
        std::vector<T> profile;  // side faces: value per cell along a
    };
    dp_source src{};
    int a = 0, p = 0, h = 0;
    long lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    long first = 0, inject = 0;
    std::vector<T> e, hf;
    std::vector<float> ge, gm, le, lm;
    T gain{}, retard{}, h_sign{};
    float sigma_e = 1, sigma_h = 1, sigma_ha = 1, sigma_ea = 1;
    float face_e[2] = {0, 0}, face_h[2] = {0, 0}, side_h[2] = {0, 0}, side_e[2] = {0, 0};
    std::vector<Face> electric_faces, magnetic_faces;

    BoxSource(const dp_source &s, const Grid &grid) : src(s) {
        a = int(s.axis);
        p = int(s.polarization);
        h = 3 - a - p;
        if (a == p) panic("a plane wave's polarization must be transverse to its travel");
        size_t l3[3], h3[3];
        grid.cell_containing(s.box_low, l3);
        grid.cell_containing(s.box_high, h3);
        for (int k = 0; k < 3; ++k) {
            lo[k] = long(l3[k]);
            hi[k] = long(h3[k]);
            if (!(lo[k] >= 1 && lo[k] < hi[k] && hi[k] + 2 <= long(grid.extent[k])))
                panic("a total-field box needs a cell of scattered field and a wall cell beyond each face");
        }
        const std::vector<float> mg_a = grid.magnetic_gains(a), eg_a = grid.electric_gains(a);
        const std::vector<float> mg_h = grid.magnetic_gains(h), eg_p = grid.electric_gains(p);
        first = lo[a] - 8;
        inject = 4;
        const long last = hi[a] + 8 + 64;
        const size_t count = size_t(last - first + 1);
        e.assign(count, T(0));
        hf.assign(count, T(0));
        ge.resize(count);
        gm.resize(count);
        le.assign(count, 0.0f);
        lm.assign(count, 0.0f);
        const long n_a = long(grid.extent[a]);
        for (size_t i = 0; i < count; ++i) {
            long c = first + long(i);
            c = c < 0 ? 0 : (c > n_a - 1 ? n_a - 1 : c);
            ge[i] = eg_a[size_t(c)];
            gm[i] = mg_a[size_t(c)];
        }
        const float t = 64.0f;
        const float peak = -(3.0f + 1.0f) * std::log(1e-6f) * grid.courant / (4.0f * t);
        const long tail0 = long(count) - 64;
        for (long i = tail0; i < long(count); ++i) {
            const float de = std::fmin(float(i - tail0 + 1) / t, 1.0f);
            const float dh = std::fmin((float(i - tail0) + 1.5f) / t, 1.0f);
            le[size_t(i)] = peak * de * de * de;
            lm[size_t(i)] = peak * dh * dh * dh;
        }
        const float spacing = grid.spacing[a].finest();
        const T dt = T(grid.time_step());
        gain = T(SPEED_OF_LIGHT * grid.time_step() / spacing);
        const T omega = T(2) * Math<T>::pi * T(s.waveform.frequency);
        retard = std::asin(Math<T>::sin(T(0.5) * omega * dt) / gain) / omega;
        h_sign = ((p + 1) % 3) == a ? T(-1) : T(1);
        sigma_e = (p + 1) % 3 == a ? 1.0f : -1.0f;
        sigma_h = (h + 1) % 3 == a ? 1.0f : -1.0f;
        sigma_ha = (a + 2) % 3 == p ? 1.0f : -1.0f;
        sigma_ea = (a + 2) % 3 == h ? 1.0f : -1.0f;
        face_e[0] = eg_a[size_t(lo[a])];
        face_e[1] = eg_a[size_t(hi[a])];
        face_h[0] = mg_a[size_t(lo[a] - 1)];
        face_h[1] = mg_a[size_t(hi[a])];
        side_h[0] = mg_h[size_t(lo[h] - 1)];
        side_h[1] = mg_h[size_t(hi[h])];
        side_e[0] = eg_p[size_t(lo[p])];
        side_e[1] = eg_p[size_t(hi[p])];
    }

    T E(long cell) const { return e[size_t(cell - first)]; }
    T H(long cell) const { return hf[size_t(cell - first)]; }

    Face face(int component, bool magnetic) const {
        Face f{};
        f.component = component;
        f.magnetic = magnetic;
        f.origin[a] = size_t(lo[a]);
        f.extent[a] = size_t(hi[a] - lo[a]);
        f.origin[p] = size_t(lo[p]);
        f.extent[p] = size_t(hi[p] - lo[p]);
        f.origin[h] = size_t(lo[h]);
        f.extent[h] = size_t(hi[h] - lo[h] + 1);
        return f;
    }

    // From the incident E at this step's start: H_h across a, H_a across h.
    void magnetic_corrections() {
        magnetic_faces.clear();
        for (int f = 0; f < 2; ++f) {
            Face c = face(h, true);
            c.origin[a] = size_t(f ? hi[a] : lo[a] - 1);
            c.extent[a] = 1;
            c.value = T(sigma_h * (f ? -face_h[1] : face_h[0])) * E(f ? hi[a] : lo[a]);
            magnetic_faces.push_back(c);
        }
        for (int f = 0; f < 2; ++f) {
            Face c = face(a, true);
            c.extent[a] = size_t(hi[a] - lo[a] + 1);
            c.origin[h] = size_t(f ? hi[h] : lo[h] - 1);
            c.extent[h] = 1;
            c.value = T(1);
            const T coef = T(sigma_ha * (f ? -side_h[1] : side_h[0]));
            for (long x = lo[a]; x <= hi[a]; ++x) c.profile.push_back(coef * E(x));
            magnetic_faces.push_back(c);
        }
    }

    // The line's H (the grid's update of a uniform wave), then its drive.
    void step_h(T time, T dt) {
        const size_t count = e.size();
        for (size_t i = 0; i < count; ++i) {
            const T next = i + 1 < count ? e[i + 1] : T(0);
            const T curl = T(sigma_h) * (T(gm[i]) * (next - e[i]));
            const T loss = T(lm[i]);
            hf[i] = loss == T(0) ? hf[i] - curl : ((T(1) - loss) * hf[i] - curl) / (T(1) + loss);
        }
        hf[size_t(inject - 1)] += h_sign * gain * (T(src.amplitude) * evaluate<T>(src.waveform, time - dt));
    }

    // From the incident H at the half step: E_p across a, E_a across p.
    void electric_corrections() {
        electric_faces.clear();
        for (int f = 0; f < 2; ++f) {
            Face c = face(p, false);
            c.origin[a] = size_t(f ? hi[a] : lo[a]);
            c.extent[a] = 1;
            c.value = T(sigma_e * (f ? face_e[1] : -face_e[0])) * H(f ? hi[a] : lo[a] - 1);
            electric_faces.push_back(c);
        }
        for (int f = 0; f < 2; ++f) {
            Face c = face(a, false);
            c.origin[p] = size_t(f ? hi[p] : lo[p]);
            c.extent[p] = 1;
            c.value = T(1);
            const T coef = T(sigma_ea * (f ? side_e[1] : -side_e[0]));
            for (long x = lo[a]; x < hi[a]; ++x) c.profile.push_back(coef * H(x));
            electric_faces.push_back(c);
        }
    }

    void step_e(T time, T dt) {
        for (size_t i = 1; i < e.size(); ++i) {
            const T curl = T(sigma_e) * (T(ge[i]) * (hf[i] - hf[i - 1]));
            const T loss = T(le[i]);
            e[i] = loss == T(0) ? e[i] + curl : ((T(1) - loss) * e[i] + curl) / (T(1) + loss);
        }
        e[size_t(inject)] += gain * (T(src.amplitude) * evaluate<T>(src.waveform, time - T(0.5) * dt + retard));
    }
};

// ---------------------------------------------------------------------------
// Simulation — src/cpu.rs:65-713
// ---------------------------------------------------------------------------
struct SimBase {
    virtual ~SimBase() = default;
};

template <typename T> struct Simulation : SimBase {
    Grid grid;
    std::vector<T> electric[3], magnetic[3];
    std::vector<uint32_t> material_index;
    std::vector<dp_material> materials;
    std::vector<Coefficients> coeff;
    std::vector<float> magnetic_gains[3], electric_gains[3];
    Absorber absorber;
    std::vector<T> intensity;
    bool accumulating = false;
    uint64_t accumulated = 0;
    std::vector<dp_source> sources;
    std::vector<std::shared_ptr<BoxSource<T>>> boxes; // per source; null unless a total-field box
    uint64_t step = 0;
    int threads = 1;

    explicit Simulation(const dp_scene_desc &d) {
        grid = Grid::build(d.grid);
        grid.validate();
        if (d.material_count == 0) panic("a material table needs vacuum at index 0");
        materials.assign(d.materials, d.materials + d.material_count);
        std::vector<dp_shape> shapes(d.shapes, d.shapes + d.shape_count);
        for (const auto &s : shapes)
            if (s.material >= d.material_count) panic("a shape refers to a missing material");
        sources.assign(d.sources, d.sources + d.source_count);
        for (const auto &src : sources)
            boxes.push_back(src.shape == DP_SOURCE_PLANE_WAVE_BOX ? std::make_shared<BoxSource<T>>(src, grid) : nullptr);
        size_t total = grid.total();
        for (int a = 0; a < 3; ++a) {
            electric[a].assign(total, T(0));
            magnetic[a].assign(total, T(0));
            magnetic_gains[a] = grid.magnetic_gains(a);
            electric_gains[a] = grid.electric_gains(a);
        }
        material_index = material_indices(grid, shapes);
        for (const auto &m : materials) coeff.push_back(coefficients(m, grid));
        intensity.assign(total, T(0));
        absorber = Absorber::build(grid, d.boundary);
    }

    T time_step() const { return T(grid.time_step()); }

    bool is_reversible() const {
        for (const auto &c : coeff)
            if (!(c.electric_loss == 0.0f && c.magnetic_loss == 0.0f)) return false;
        return absorber.peak() == 0.0f;
    }

    void reset() {
        for (int a = 0; a < 3; ++a) {
            std::fill(electric[a].begin(), electric[a].end(), T(0));
            std::fill(magnetic[a].begin(), magnetic[a].end(), T(0));
        }
        std::fill(intensity.begin(), intensity.end(), T(0));
        accumulated = 0;
        step = 0;
        for (auto &b : boxes)
            if (b) b = std::make_shared<BoxSource<T>>(b->src, grid);
    }

    // src/cpu.rs:174-198
    void advance() {
        // `(step + 1) as f32 * time_step()` in f32; exact in the f64 instance.
        T time = std::is_same_v<T, float> ? T(static_cast<float>(step + 1) * grid.time_step())
                                          : T(double(step + 1) * double(grid.time_step()));
        const T dt = T(grid.time_step());
        for (auto &b : boxes)
            if (b) b->magnetic_corrections();
        update_magnetic(false);
        apply_sources(time, T(1), true);
        for (auto &b : boxes)
            if (b) {
                b->step_h(time, dt);
                b->electric_corrections();
            }
        update_electric(false);
        apply_sources(time, T(1), false);
        for (auto &b : boxes)
            if (b) b->step_e(time, dt);
        if (accumulating) {
            const long n = long(intensity.size());
#pragma omp parallel for schedule(static) num_threads(threads)
            for (long i = 0; i < n; ++i) {
                T sum = T(0);
                for (int a = 0; a < 3; ++a) sum += electric[a][i] * electric[a][i];
                intensity[i] += sum;
            }
            accumulated += 1;
        }
        step += 1;
    }

    // src/cpu.rs:253-273
    void reverse() {
        for (const auto &b : boxes)
            if (b) panic("a total-field box's incident line absorbs at its far end, so it does not run backwards");
        if (!is_reversible()) panic("this scene is lossy, and running a dissipative update backwards amplifies roundoff");
        if (step == 0) panic("cannot step back past the start");
        clear_intensity();
        T time = std::is_same_v<T, float> ? T(static_cast<float>(step) * grid.time_step())
                                          : T(double(step) * double(grid.time_step()));
        apply_sources(time, T(-1), false);
        update_electric(true);
        apply_sources(time, T(-1), true);
        update_magnetic(true);
        step -= 1;
    }

    // One H cell update: forward (src/cpu.rs:328-330) or its inverse (:529-531).
    static inline T h_cell(T target, T loss, T gain, T curl, bool reverse) {
        if (!reverse) return ((T(1) - loss) * target - gain * curl) / (T(1) + loss);
        return ((T(1) + loss) * target + gain * curl) / (T(1) - loss);
    }
    static inline T e_cell(T target, T loss, T gain, T curl, bool reverse) {
        if (!reverse) return ((T(1) - loss) * target + gain * curl) / (T(1) + loss);
        return ((T(1) + loss) * target - gain * curl) / (T(1) - loss);
    }

    // update_magnetic — src/cpu.rs:283-376; reverse_magnetic — :490-572.
    void update_magnetic(bool reverse) {
        const size_t ext[3] = {grid.extent[0], grid.extent[1], grid.extent[2]};
        const size_t strides[3] = {1, ext[0], ext[0] * ext[1]};
        for (int a = 0; a < 3; ++a) {
            int b = (a + 1) % 3, c = (a + 2) % 3;
            size_t stride_b = strides[b], stride_c = strides[c];
            size_t limit[3] = {ext[0], ext[1], ext[2]};
            limit[b] -= 1;
            limit[c] -= 1;
            const auto &gain_b = magnetic_gains[b];
            const auto &gain_c = magnetic_gains[c];
            T *target = magnetic[a].data();
            const T *field_b = electric[b].data();
            const T *field_c = electric[c].data();
            const auto &ax = absorber.pick(false, a, 0);
            const auto &ay = absorber.pick(false, a, 1);
            const auto &az = absorber.pick(false, a, 2);
            const long lz = long(limit[2]);
#pragma omp parallel for schedule(static) num_threads(threads)
            for (long zz = 0; zz < lz; ++zz) {
                size_t z = size_t(zz);
                for (size_t y = 0; y < limit[1]; ++y) {
                    size_t row = (z * ext[1] + y) * ext[0];
                    float absorb_row = ay[y] + az[z];
                    size_t along_row[3] = {0, y, z};
                    float row_b = b == 0 ? 1.0f : gain_b[along_row[b]];
                    float row_c = c == 0 ? 1.0f : gain_c[along_row[c]];
                    for (size_t x = 0; x < limit[0]; ++x) {
                        size_t index = row + x;
                        float gbx = b == 0 ? gain_b[x] : 1.0f;
                        float gcx = c == 0 ? gain_c[x] : 1.0f;
                        T gb = T(row_b * gbx), gc = T(row_c * gcx);
                        T curl = gb * (field_c[index + stride_b] - field_c[index]) -
                                 gc * (field_b[index + stride_c] - field_b[index]);
                        const Coefficients &k = coeff[material_index[index]];
                        T loss = T(k.magnetic_loss + absorb_row + ax[x]);
                        target[index] = h_cell(target[index], loss, T(k.magnetic_gain), curl, reverse);
                    }
                }
            }
            // High-wall planes (src/cpu.rs:343-374), implicit zero beyond the wall.
            size_t last_b = ext[b] - 1, last_c = ext[c] - 1;
            struct Wall { int fixed; size_t at; size_t others; };
            Wall walls[2] = {{b, last_b, ext[c]}, {c, last_c, last_b}};
            for (const Wall &wall : walls) {
                int other = b + c - wall.fixed;
                const long others = long(wall.others);
#pragma omp parallel for schedule(static) num_threads(threads)
                for (long ww = 0; ww < others; ++ww) {
                    for (size_t v = 0; v < ext[a]; ++v) {
                        size_t coord[3] = {0, 0, 0};
                        coord[wall.fixed] = wall.at;
                        coord[other] = size_t(ww);
                        coord[a] = v;
                        size_t index = (coord[2] * ext[1] + coord[1]) * ext[0] + coord[0];
                        T next_c = coord[b] + 1 < ext[b] ? field_c[index + stride_b] : T(0);
                        T next_b = coord[c] + 1 < ext[c] ? field_b[index + stride_c] : T(0);
                        T curl = T(gain_b[coord[b]]) * (next_c - field_c[index]) -
                                 T(gain_c[coord[c]]) * (next_b - field_b[index]);
                        float absorb_row = ay[coord[1]] + az[coord[2]];
                        const Coefficients &k = coeff[material_index[index]];
                        T loss = T(k.magnetic_loss + absorb_row + ax[coord[0]]);
                        target[index] = h_cell(target[index], loss, T(k.magnetic_gain), curl, reverse);
                    }
                }
            }
        }
    }

    // update_electric — src/cpu.rs:380-434; reverse_electric — :441-487.
    void update_electric(bool reverse) {
        const size_t ext[3] = {grid.extent[0], grid.extent[1], grid.extent[2]};
        const size_t strides[3] = {1, ext[0], ext[0] * ext[1]};
        for (int a = 0; a < 3; ++a) {
            int b = (a + 1) % 3, c = (a + 2) % 3;
            size_t stride_b = strides[b], stride_c = strides[c];
            size_t start[3] = {0, 0, 0};
            start[b] = 1;
            start[c] = 1;
            const auto &gain_b = electric_gains[b];
            const auto &gain_c = electric_gains[c];
            T *target = electric[a].data();
            const T *field_b = magnetic[b].data();
            const T *field_c = magnetic[c].data();
            const auto &ax = absorber.pick(true, a, 0);
            const auto &ay = absorber.pick(true, a, 1);
            const auto &az = absorber.pick(true, a, 2);
            const long z0 = long(start[2]), z1 = long(ext[2]);
#pragma omp parallel for schedule(static) num_threads(threads)
            for (long zz = z0; zz < z1; ++zz) {
                size_t z = size_t(zz);
                for (size_t y = start[1]; y < ext[1]; ++y) {
                    size_t row = (z * ext[1] + y) * ext[0];
                    float absorb_row = ay[y] + az[z];
                    size_t along_row[3] = {0, y, z};
                    float row_b = b == 0 ? 1.0f : gain_b[along_row[b]];
                    float row_c = c == 0 ? 1.0f : gain_c[along_row[c]];
                    for (size_t x = start[0]; x < ext[0]; ++x) {
                        size_t index = row + x;
                        float gbx = b == 0 ? gain_b[x] : 1.0f;
                        float gcx = c == 0 ? gain_c[x] : 1.0f;
                        T gb = T(row_b * gbx), gc = T(row_c * gcx);
                        T curl = gb * (field_c[index] - field_c[index - stride_b]) -
                                 gc * (field_b[index] - field_b[index - stride_c]);
                        const Coefficients &k = coeff[material_index[index]];
                        T loss = T(k.electric_loss + absorb_row + ax[x]);
                        target[index] = e_cell(target[index], loss, T(k.electric_gain), curl, reverse);
                    }
                }
            }
        }
    }

    void set_accumulate_intensity(bool on) {
        if (on && !accumulating) clear_intensity();
        accumulating = on;
    }
    void clear_intensity() {
        if (accumulated > 0) {
            std::fill(intensity.begin(), intensity.end(), T(0));
            accumulated = 0;
        }
    }

    // apply_sources — src/cpu.rs:606-633
    void apply_sources(T time, T sign, bool magnetic_phase) {
        for (size_t k = 0; k < sources.size(); ++k) {
            const dp_source &source = sources[k];
            if (boxes[k]) {
                apply_box(*boxes[k], magnetic_phase);
                continue;
            }
            Injection<T> inj[2];
            injections<T>(source, grid, time, inj);
            for (const auto &injection : inj) {
                if (injection.value == T(0) || injection.magnetic != magnetic_phase) continue;
                T value = sign * injection.value;
                T *target = injection.magnetic ? magnetic[injection.component].data()
                                               : electric[injection.component].data();
                for (size_t dz = 0; dz < injection.extent[2]; ++dz)
                    for (size_t dy = 0; dy < injection.extent[1]; ++dy)
                        for (size_t dx = 0; dx < injection.extent[0]; ++dx) {
                            size_t coord[3] = {injection.origin[0] + dx, injection.origin[1] + dy,
                                               injection.origin[2] + dz};
                            float position[3];
                            grid.cell_center(coord, position);
                            target[grid.index(coord[0], coord[1], coord[2])] +=
                                value * T(injection.weight(position));
                        }
            }
        }
    }

    // Total-field boxes' incident lines brought to `target` steps from the
    // start (their state depends on the step count alone).
    void seek_boxes(uint64_t target) {
        const T dt = T(grid.time_step());
        for (auto &b : boxes) {
            if (!b) continue;
            b = std::make_shared<BoxSource<T>>(b->src, grid);
            for (uint64_t n = 0; n < target; ++n) {
                const T time = std::is_same_v<T, float> ? T(static_cast<float>(n + 1) * grid.time_step())
                                                        : T(double(n + 1) * double(grid.time_step()));
                b->step_h(time, dt);
                b->step_e(time, dt);
            }
        }
    }

    // A box's corrections of one phase: a uniform face adds value · 1 (skipped
    // when zero, as any injection), a side face its profile value · 1.
    void apply_box(const BoxSource<T> &b, bool magnetic_phase) {
        for (const auto &f : magnetic_phase ? b.magnetic_faces : b.electric_faces) {
            if (f.profile.empty() && f.value == T(0)) continue;
            T *target = f.magnetic ? magnetic[f.component].data() : electric[f.component].data();
            for (size_t dz = 0; dz < f.extent[2]; ++dz)
                for (size_t dy = 0; dy < f.extent[1]; ++dy)
                    for (size_t dx = 0; dx < f.extent[0]; ++dx) {
                        const size_t c[3] = {f.origin[0] + dx, f.origin[1] + dy, f.origin[2] + dz};
                        const T w = f.profile.empty() ? T(1.0f) : f.profile[c[b.a] - f.origin[b.a]];
                        target[grid.index(c[0], c[1], c[2])] += f.value * w;
                    }
        }
    }

    // energy_density — src/cpu.rs:689-703: per cell, summed over both fields.
    void energy_density(float *out) const {
        const size_t n = grid.total();
        for (size_t i = 0; i < n; ++i) {
            float density = 0.0f;
            for (int a = 0; a < 3; ++a) {
                const float e = float(electric[a][i]), h = float(magnetic[a][i]);
                density += 0.5f * (e * e + h * h);
            }
            out[i] = density;
        }
    }

    // energy — src/cpu.rs:654-687
    void energy(double *electric_out, double *magnetic_out) const {
        const size_t ext[3] = {grid.extent[0], grid.extent[1], grid.extent[2]};
        double ee = 0.0, em = 0.0;
        for (size_t z = 0; z < ext[2]; ++z)
            for (size_t y = 0; y < ext[1]; ++y) {
                size_t row = (z * ext[1] + y) * ext[0];
                for (size_t x = 0; x < ext[0]; ++x) {
                    size_t index = row + x;
                    size_t coord[3] = {x, y, z};
                    const dp_material &m = materials[material_index[index]];
                    for (int a = 0; a < 3; ++a) {
                        int b = (a + 1) % 3, c = (a + 2) % 3;
                        T e = electric[a][index];
                        T h = magnetic[a][index];
                        double ev = double(grid.spacing[a].primary[coord[a]]) *
                                    double(grid.spacing[b].dual[coord[b]]) *
                                    double(grid.spacing[c].dual[coord[c]]);
                        double mv = double(grid.spacing[a].dual[coord[a]]) *
                                    double(grid.spacing[b].primary[coord[b]]) *
                                    double(grid.spacing[c].primary[coord[c]]);
                        ee += 0.5 * ev * double(T(m.relative_permittivity) * e * e);
                        em += 0.5 * mv * double(T(m.relative_permeability) * h * h);
                    }
                }
            }
        *electric_out = ee;
        *magnetic_out = em;
    }

    bool is_finite() const {
        for (int a = 0; a < 3; ++a) {
            for (T v : electric[a]) if (!std::isfinite(v)) return false;
            for (T v : magnetic[a]) if (!std::isfinite(v)) return false;
        }
        return true;
    }
};

} // namespace oracle

// ---------------------------------------------------------------------------
// C interface for the test harness (ctypes).
// ---------------------------------------------------------------------------
using namespace oracle;

struct or_sim {
    Simulation<float> *f32 = nullptr;
    Simulation<double> *f64 = nullptr;
};

#define OR_TRY(...)                                                                    \
    try {                                                                              \
        __VA_ARGS__;                                                                   \
    } catch (const Panic &p) {                                                         \
        last_error = p.message;                                                        \
        return 1;                                                                      \
    } catch (const std::exception &e) {                                                \
        last_error = e.what();                                                         \
        return 1;                                                                      \
    }

template <typename T> static int read_field_t(Simulation<T> *sim, int field, double *out64, float *out32) {
    size_t n = sim->grid.total();
    if (field == DP_FIELD_INTENSITY) {
        for (size_t i = 0; i < n; ++i) {
            if (out64) out64[i] = double(sim->intensity[i]);
            if (out32) out32[i] = float(sim->intensity[i]);
        }
        return 0;
    }
    auto &f = field == DP_FIELD_ELECTRIC ? sim->electric : sim->magnetic;
    for (int a = 0; a < 3; ++a)
        for (size_t i = 0; i < n; ++i) {
            if (out64) out64[a * n + i] = double(f[a][i]);
            if (out32) out32[a * n + i] = float(f[a][i]);
        }
    return 0;
}

extern "C" {

const char *or_last_error(void) { return last_error.c_str(); }

int or_sim_create(const dp_scene_desc *desc, int fp64, or_sim **out) {
    OR_TRY({
        auto *s = new or_sim();
        if (fp64) s->f64 = new Simulation<double>(*desc);
        else s->f32 = new Simulation<float>(*desc);
        *out = s;
        return 0;
    });
}

void or_sim_destroy(or_sim *s) {
    if (!s) return;
    delete s->f32;
    delete s->f64;
    delete s;
}

void or_sim_set_threads(or_sim *s, int threads) {
    if (s->f32) s->f32->threads = threads;
    if (s->f64) s->f64->threads = threads;
}

int or_sim_advance(or_sim *s, uint64_t steps) {
    OR_TRY({
        for (uint64_t i = 0; i < steps; ++i) {
            if (s->f32) s->f32->advance();
            else s->f64->advance();
        }
        return 0;
    });
}

int or_sim_reverse(or_sim *s, uint64_t steps) {
    OR_TRY({
        for (uint64_t i = 0; i < steps; ++i) {
            if (s->f32) s->f32->reverse();
            else s->f64->reverse();
        }
        return 0;
    });
}

void or_sim_reset(or_sim *s) {
    if (s->f32) s->f32->reset();
    else s->f64->reset();
}

uint64_t or_sim_step_count(const or_sim *s) { return s->f32 ? s->f32->step : s->f64->step; }

float or_sim_time(const or_sim *s) {
    uint64_t step = or_sim_step_count(s);
    const Grid &g = s->f32 ? s->f32->grid : s->f64->grid;
    return static_cast<float>(step) * g.time_step();
}

int or_sim_is_reversible(const or_sim *s) { return s->f32 ? s->f32->is_reversible() : s->f64->is_reversible(); }

void or_sim_set_accumulate_intensity(or_sim *s, int on) {
    if (s->f32) s->f32->set_accumulate_intensity(on != 0);
    else s->f64->set_accumulate_intensity(on != 0);
}

uint64_t or_sim_accumulated_steps(const or_sim *s) { return s->f32 ? s->f32->accumulated : s->f64->accumulated; }

int or_sim_read_field(or_sim *s, int field, float *out) {
    return s->f32 ? read_field_t(s->f32, field, nullptr, out) : read_field_t(s->f64, field, nullptr, out);
}
int or_sim_read_field64(or_sim *s, int field, double *out) {
    return s->f32 ? read_field_t(s->f32, field, out, nullptr) : read_field_t(s->f64, field, out, nullptr);
}

int or_sim_write_field(or_sim *s, int field, const float *in) {
    if (s->f32) {
        size_t n = s->f32->grid.total();
        auto &f = field == DP_FIELD_ELECTRIC ? s->f32->electric : s->f32->magnetic;
        for (int a = 0; a < 3; ++a) std::memcpy(f[a].data(), in + a * n, n * sizeof(float));
    } else {
        size_t n = s->f64->grid.total();
        auto &f = field == DP_FIELD_ELECTRIC ? s->f64->electric : s->f64->magnetic;
        for (int a = 0; a < 3; ++a)
            for (size_t i = 0; i < n; ++i) f[a][i] = double(in[a * n + i]);
    }
    return 0;
}

// Steppable::restore (src/cpu.rs:737-752): intensity cleared, fields copied,
// the step rewound.
int or_sim_restore(or_sim *s, uint64_t step, const float *electric, const float *magnetic) {
    auto restore = [&](auto *sim) {
        sim->clear_intensity();
        size_t n = sim->grid.total();
        for (int a = 0; a < 3; ++a)
            for (size_t i = 0; i < n; ++i) {
                sim->electric[a][i] = electric[a * n + i];
                sim->magnetic[a][i] = magnetic[a * n + i];
            }
        sim->step = step;
        sim->seek_boxes(step);
    };
    if (s->f32) restore(s->f32);
    else restore(s->f64);
    return 0;
}

// One value, or one component, of a field (sample_electric and friends,
// src/cpu.rs:136-160).
float or_sim_sample(const or_sim *s, int field, int component, uint32_t x, uint32_t y, uint32_t z) {
    auto sample = [&](auto *sim) -> float {
        size_t i = sim->grid.index(x, y, z);
        if (field == DP_FIELD_INTENSITY) return float(sim->intensity[i]);
        auto &f = field == DP_FIELD_ELECTRIC ? sim->electric : sim->magnetic;
        return float(f[component][i]);
    };
    return s->f32 ? sample(s->f32) : sample(s->f64);
}

int or_sim_component(const or_sim *s, int field, int component, float *out) {
    auto read = [&](auto *sim) {
        size_t n = sim->grid.total();
        auto &f = field == DP_FIELD_ELECTRIC ? sim->electric : sim->magnetic;
        for (size_t i = 0; i < n; ++i) out[i] = float(f[component][i]);
    };
    if (s->f32) read(s->f32);
    else read(s->f64);
    return 0;
}

void or_sim_energy(const or_sim *s, double *electric, double *magnetic) {
    if (s->f32) s->f32->energy(electric, magnetic);
    else s->f64->energy(electric, magnetic);
}

int or_sim_is_finite(const or_sim *s) { return s->f32 ? s->f32->is_finite() : s->f64->is_finite(); }

// Scene::energy_density of the f32 instance.
int or_sim_energy_density(const or_sim *s, float *out) {
    if (!s->f32) return 1;
    s->f32->energy_density(out);
    return 0;
}

void or_sim_extent(const or_sim *s, uint32_t out[3]) {
    const Grid &g = s->f32 ? s->f32->grid : s->f64->grid;
    for (int a = 0; a < 3; ++a) out[a] = g.extent[a];
}

float or_sim_time_step(const or_sim *s) { return (s->f32 ? s->f32->grid : s->f64->grid).time_step(); }

// Setup tables, in the same packing as dp_scene_table.
int or_sim_table(const or_sim *s, int table, void *out) {
    if (!s->f32) return 1;
    const Simulation<float> &sim = *s->f32;
    const Grid &g = sim.grid;
    float *f = static_cast<float *>(out);
    size_t k = 0;
    switch (table) {
    case DP_TABLE_MAGNETIC_GAINS:
        for (int a = 0; a < 3; ++a) for (float v : sim.magnetic_gains[a]) f[k++] = v;
        return 0;
    case DP_TABLE_ELECTRIC_GAINS:
        for (int a = 0; a < 3; ++a) for (float v : sim.electric_gains[a]) f[k++] = v;
        return 0;
    case DP_TABLE_CELL_CENTERS:
        for (int a = 0; a < 3; ++a) for (float v : g.cell_centers(a)) f[k++] = v;
        return 0;
    case DP_TABLE_ABSORBER:
        for (int a = 0; a < 3; ++a) for (float v : sim.absorber.integer[a]) f[k++] = v;
        for (int a = 0; a < 3; ++a) for (float v : sim.absorber.half[a]) f[k++] = v;
        return 0;
    case DP_TABLE_COEFFICIENTS:
        for (const auto &c : sim.coeff) {
            f[k++] = c.electric_gain; f[k++] = c.electric_loss;
            f[k++] = c.magnetic_gain; f[k++] = c.magnetic_loss;
        }
        return 0;
    case DP_TABLE_MATERIAL_INDEX: {
        uint32_t *u = static_cast<uint32_t *>(out);
        std::memcpy(u, sim.material_index.data(), sim.material_index.size() * sizeof(uint32_t));
        return 0;
    }
    case DP_TABLE_PRIMARY:
        for (int a = 0; a < 3; ++a) for (float v : g.spacing[a].primary) f[k++] = v;
        return 0;
    case DP_TABLE_DUAL:
        for (int a = 0; a < 3; ++a) for (float v : g.spacing[a].dual) f[k++] = v;
        return 0;
    }
    return 1;
}

float or_sim_absorber_peak(const or_sim *s) { return (s->f32 ? s->f32->absorber : s->f64->absorber).peak(); }

// Source::injections at a time, for the source unit tests (f32 instance).
int or_sim_injections(const or_sim *s, float time, dp_injection *out, uint32_t capacity, uint32_t *count) {
    if (!s->f32) return 1;
    const auto &sim = *s->f32;
    uint32_t n = 0;
    for (const auto &src : sim.sources) {
        if (src.shape == DP_SOURCE_PLANE_WAVE_BOX) return 1; // depends on its line's history, not on time alone
        Injection<float> inj[2];
        injections<float>(src, sim.grid, time, inj);
        for (const auto &i : inj) {
            if (n >= capacity) return 1;
            dp_injection &o = out[n++];
            for (int a = 0; a < 3; ++a) {
                o.origin[a] = uint32_t(i.origin[a]);
                o.extent[a] = uint32_t(i.extent[a]);
                o.center[a] = i.center[a];
            }
            o.component = uint32_t(i.component);
            o.magnetic = i.magnetic ? 1 : 0;
            o.value = i.value;
            o.inverse_waist_squared = i.inverse_waist_squared;
        }
    }
    *count = n;
    return 0;
}

// Apodization weight of one injection at a position (src/source.rs:441-455).
float or_injection_weight(const dp_injection *inj, const float position[3]) {
    Injection<float> i{};
    for (int a = 0; a < 3; ++a) {
        i.extent[a] = inj->extent[a];
        i.center[a] = inj->center[a];
    }
    i.inverse_waist_squared = inj->inverse_waist_squared;
    return i.weight(position);
}

// Grid-level helpers for the grid unit tests.
int or_grid_resolve(const dp_grid_spec *spec, uint32_t extent_out[3], float *time_step, float *worst_ratio,
                    float *finest, float *coarsest, float size_out[3]) {
    OR_TRY({
        Grid g = Grid::build(*spec);
        float worst = 1.0f;
        for (int a = 0; a < 3; ++a) {
            extent_out[a] = g.extent[a];
            size_out[a] = g.size(a);
            worst = std::fmax(worst, g.spacing[a].worst_ratio());
        }
        *time_step = g.time_step();
        *worst_ratio = worst;
        *finest = g.finest();
        *coarsest = g.coarsest();
        return 0;
    });
}

// The resolved grid in the C ABI's own dp_grid_info layout, so that a caller
// building scenes on the CPU alone (the timed CPU baseline) needs no other
// library: Grid::{extent, size, time_step, finest, coarsest,
// reference_cell_size} (src/grid.rs:521-594).
int or_grid_info(const dp_grid_spec *spec, dp_grid_info *out) {
    OR_TRY({
        Grid g = Grid::build(*spec);
        float worst = 1.0f;
        for (int a = 0; a < 3; ++a) {
            out->extent[a] = g.extent[a];
            out->size[a] = g.size(a);
            worst = std::fmax(worst, g.spacing[a].worst_ratio());
        }
        out->time_step = g.time_step();
        out->finest = g.finest();
        out->coarsest = g.coarsest();
        out->worst_ratio = worst;
        out->reference_cell_size = g.reference_cell_size();
        return 0;
    });
}

// to_cell / to_position / cell_containing / cell_center through a grid.
int or_grid_map(const dp_grid_spec *spec, int op, const float in[3], float out[3]) {
    OR_TRY({
        Grid g = Grid::build(*spec);
        if (op == 0) {
            for (int a = 0; a < 3; ++a) out[a] = g.spacing[a].coordinate(in[a]);
        } else if (op == 1) {
            for (int a = 0; a < 3; ++a) out[a] = g.spacing[a].position(in[a]);
        } else if (op == 2) {
            size_t c[3];
            g.cell_containing(in, c);
            for (int a = 0; a < 3; ++a) out[a] = float(c[a]);
        } else {
            size_t c[3] = {size_t(in[0]), size_t(in[1]), size_t(in[2])};
            g.cell_center(c, out);
        }
        return 0;
    });
}

float or_numerical_phase_velocity(float courant, float cells, const float direction[3]) {
    return numerical_phase_velocity(courant, cells, direction);
}

float or_waveform_evaluate(const dp_waveform *w, float time) { return evaluate<float>(*w, time); }

int or_max_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

} // extern "C"
