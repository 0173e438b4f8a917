// Host-side scene resolution.  See setup.hpp.
//
// Arithmetic follows the reference's f32 expressions in their evaluation
// order (Rust never contracts to FMA; this file is compiled with
// -ffp-contract=off), so the tables uploaded to the device are the ones the
// reference's own solvers would hold.
#include "setup.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <limits>

namespace diaphane {

namespace {

[[noreturn]] void invalid(const std::string &m) { throw Error(DP_ERR_INVALID, m); }

// Rust `as` casts from f32 saturate at the target range.
size_t to_index(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 1.8446744e19f) return SIZE_MAX;
    return size_t(v);
}
uint32_t to_u32(float v) {
    if (!(v > 0.0f)) return 0;
    if (v >= 4294967296.0f) return UINT32_MAX;
    return uint32_t(v);
}

Axis1D assemble(std::vector<float> primary, std::vector<float> corners) {
    // Spacing::assemble, src/grid.rs:192-214.
    if (primary.size() < 2) invalid("an axis needs at least 2 cells");
    for (float w : primary)
        if (!(w > 0.0f && std::isfinite(w))) invalid("cell widths must be positive and finite");
    Axis1D axis;
    axis.dual.resize(primary.size());
    axis.dual[0] = 0.5f * (primary[0] + primary[0]);
    for (size_t i = 1; i < primary.size(); ++i) axis.dual[i] = 0.5f * (primary[i - 1] + primary[i]);
    axis.primary = std::move(primary);
    axis.corners = std::move(corners);
    return axis;
}

} // namespace

float Axis1D::finest() const {
    float m = std::numeric_limits<float>::infinity();
    for (float w : primary) m = std::fmin(m, w);
    return m;
}

float Axis1D::coarsest() const {
    float m = -std::numeric_limits<float>::infinity();
    for (float w : primary) m = std::fmax(m, w);
    return m;
}

float Axis1D::worst_ratio() const {
    float m = 1.0f;
    for (size_t i = 1; i < primary.size(); ++i)
        m = std::fmax(m, std::fmax(primary[i] / primary[i - 1], primary[i - 1] / primary[i]));
    return m;
}

// Spacing::position / offset_of, src/grid.rs:262-285.
float Axis1D::position(float coordinate) const {
    size_t last = primary.size() - 1;
    size_t i = std::min(to_index(std::fmax(std::floor(coordinate), 0.0f)), last);
    float offset = corners[i] + (coordinate - float(i)) * primary[i];
    return offset - 0.5f * length();
}

// Spacing::coordinate, src/grid.rs:269-279: a search, not a division.
float Axis1D::coordinate(float position) const {
    float offset = position + 0.5f * length();
    size_t first_past = size_t(std::upper_bound(corners.begin(), corners.end(), offset) - corners.begin());
    size_t i = first_past == 0 ? 0 : first_past - 1;
    if (i > primary.size() - 1) i = primary.size() - 1;
    return float(i) + (offset - corners[i]) / primary[i];
}

// Spacing::uniform, src/grid.rs:167-178: corners by f64 multiplication.
Axis1D axis_uniform(uint32_t count, float width) {
    if (count < 2) invalid("an axis needs at least 2 cells");
    std::vector<float> corners(size_t(count) + 1);
    for (uint32_t i = 0; i <= count; ++i) corners[i] = float(double(i) * double(width));
    return assemble(std::vector<float>(count, width), std::move(corners));
}

// Spacing::from_widths, src/grid.rs:181-190: corners by an f64 running sum.
Axis1D axis_from_widths(std::vector<float> widths) {
    std::vector<float> corners(widths.size() + 1);
    double sum = 0.0;
    corners[0] = 0.0f;
    for (size_t i = 0; i < widths.size(); ++i) {
        sum += double(widths[i]);
        corners[i + 1] = float(sum);
    }
    return assemble(std::move(widths), std::move(corners));
}

// grade(), src/grid.rs:791-888: sample the target width, cap its slope with a
// forward and a backward sweep, march the cells, re-cap them, drop the last
// cell if that lands nearer the wall, then rescale onto the wall.
Axis1D axis_graded(int axis, float length, float base, const dp_refinement *refinements,
                   uint32_t refinement_count, float max_ratio) {
    std::vector<const dp_refinement *> active;
    for (uint32_t i = 0; i < refinement_count; ++i)
        if (refinements[i].size[axis] > 0.0f) active.push_back(&refinements[i]);
    if (active.empty()) return axis_uniform(to_u32(std::fmax(std::round(length / base), 2.0f)), base);

    float finest = base;
    for (const dp_refinement *r : active) finest = std::fmin(finest, r->cell_size);
    if (!(finest > 0.0f && std::isfinite(finest))) invalid("refinement cell sizes must be positive and finite");

    size_t samples = to_index(std::ceil(length / finest * 4.0f));
    samples = std::max<size_t>(64, std::min<size_t>(samples, size_t(1) << 20));
    const float step = length / float(samples);

    std::vector<float> target(samples + 1);
    for (size_t i = 0; i <= samples; ++i) {
        float position = float(i) * step - 0.5f * length;
        float width = base;
        for (const dp_refinement *r : active) {
            float half = 0.5f * r->size[axis];
            if (std::fabs(position - r->center[axis]) <= half) width = std::fmin(width, r->cell_size);
        }
        target[i] = width;
    }
    const float slope = (max_ratio - 1.0f) * step;
    for (size_t i = 1; i <= samples; ++i) target[i] = std::fmin(target[i], target[i - 1] + slope);
    for (size_t i = samples; i-- > 0;) target[i] = std::fmin(target[i], target[i + 1] + slope);

    std::vector<float> widths;
    for (float offset = 0.0f; offset < length;) {
        size_t i = std::min(to_index(offset / step), samples);
        widths.push_back(target[i]);
        offset += target[i];
        if (widths.size() > (size_t(1) << 16)) invalid("grading ran to more cells than an axis can carry");
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
    const float scale = length / total;
    for (float &w : widths) w *= scale;
    return axis_from_widths(std::move(widths));
}

// Grid::build, src/grid.rs:466-508.
ResolvedGrid ResolvedGrid::build(const dp_grid_spec &spec) {
    if (!(spec.cell_size > 0.0f && std::isfinite(spec.cell_size))) invalid("cell size must be positive and finite");
    if (!(spec.max_ratio > 1.0f && std::isfinite(spec.max_ratio))) invalid("the growth cap must exceed 1");
    if (spec.refinement_count > 0 && spec.refinements == nullptr) invalid("refinements pointer is null");
    ResolvedGrid g;
    for (int a = 0; a < 3; ++a) {
        if (spec.refinement_count == 0)
            g.axes[a] = axis_uniform(spec.extent[a], spec.cell_size);
        else
            g.axes[a] = axis_graded(a, float(spec.extent[a]) * spec.cell_size, spec.cell_size, spec.refinements,
                                    spec.refinement_count, spec.max_ratio);
        g.n[a] = uint32_t(g.axes[a].primary.size());
    }
    g.courant = spec.courant;
    g.base = spec.cell_size;
    return g;
}

// Grid::validate, src/grid.rs:747-773.
void ResolvedGrid::validate() const {
    for (int a = 0; a < 3; ++a)
        if (n[a] < 2) invalid("grid must be at least 2 cells across on every axis");
    if (!(courant > 0.0f && courant <= kCourantLimit)) invalid("Courant number is outside (0, 1/sqrt(3)]; the scheme would diverge");
}

// src/grid.rs:575-584.
float ResolvedGrid::reference_cell_size() const {
    float inverse_squares = 0.0f;
    for (int a = 0; a < 3; ++a) {
        float f = axes[a].finest();
        inverse_squares += 1.0f / (f * f);
    }
    return std::sqrt(3.0f / inverse_squares);
}

float ResolvedGrid::time_step() const { return courant * reference_cell_size() / kSpeedOfLight; }

float ResolvedGrid::finest() const {
    float m = std::numeric_limits<float>::infinity();
    for (int a = 0; a < 3; ++a) m = std::fmin(m, axes[a].finest());
    return m;
}

float ResolvedGrid::coarsest() const {
    float m = -std::numeric_limits<float>::infinity();
    for (int a = 0; a < 3; ++a) m = std::fmax(m, axes[a].coarsest());
    return m;
}

void ResolvedGrid::cell_center(const uint32_t coord[3], float out[3]) const {
    for (int a = 0; a < 3; ++a) out[a] = axes[a].position(float(coord[a]) + 0.5f);
}

void ResolvedGrid::cell_containing(const float position[3], uint32_t out[3]) const {
    for (int a = 0; a < 3; ++a) {
        float c = axes[a].coordinate(position[a]);
        size_t i = to_index(std::fmax(std::floor(c), 0.0f));
        out[a] = uint32_t(std::min<size_t>(i, n[a] - 1));
    }
}

bool ResolvedGrid::contains(const float position[3]) const {
    for (int a = 0; a < 3; ++a)
        if (!(std::fabs(position[a]) <= 0.5f * axes[a].length())) return false;
    return true;
}

template <typename T> constexpr T pi_in();
template <> constexpr float pi_in<float>() { return kPi; }
template <> constexpr double pi_in<double>() { return 3.14159265358979323846; }

// Waveform::evaluate, src/source.rs:74-115.
template <typename T> T waveform_in(const dp_waveform &w, T t) {
    const T pi = pi_in<T>();
    switch (w.kind) {
    case DP_WAVE_RICKER: {
        T arg = pi * T(w.frequency) * (t - T(w.delay));
        T arg2 = arg * arg;
        return (T(1) - T(2) * arg2) * std::exp(-arg2);
    }
    case DP_WAVE_GAUSSIAN_PULSE: {
        const T fwhm_to_sigma = T(0.4246609f); // 1 / (2 sqrt(2 ln 2))
        T sigma = fwhm_to_sigma * T(w.duration_cycles) / T(w.frequency);
        T tau = t - T(w.delay);
        T envelope = std::exp(T(-0.5) * (tau / sigma) * (tau / sigma));
        return envelope * std::sin(T(2) * pi * T(w.frequency) * tau);
    }
    case DP_WAVE_CONTINUOUS: {
        if (t <= T(0)) return T(0);
        T ramp = T(w.ramp_cycles) / T(w.frequency);
        T envelope = t >= ramp ? T(1) : T(0.5) * (T(1) - std::cos(pi * t / ramp));
        return envelope * std::sin(T(2) * pi * T(w.frequency) * t);
    }
    }
    return T(0);
}
template float waveform_in<float>(const dp_waveform &, float);
template double waveform_in<double>(const dp_waveform &, double);

// Injection::weight, src/source.rs:441-455.
float injection_weight(const StepInjection &inj, const float position[3]) {
    if (inj.inverse_waist_squared == 0.0f) return 1.0f;
    float r2 = 0.0f;
    for (int a = 0; a < 3; ++a)
        if (inj.extent[a] > 1) {
            float d = position[a] - inj.center[a];
            r2 += d * d;
        }
    return std::exp(-r2 * inj.inverse_waist_squared);
}

namespace {

// Material::coefficients, src/material.rs:100-122.
Coeff material_coefficients(const dp_material &m, float dt) {
    if (std::isinf(m.conductivity)) return Coeff{0.0f, 1.0f, 1.0f / m.relative_permeability, 0.0f};
    float half_step = 0.5f * dt;
    return Coeff{1.0f / m.relative_permittivity,
                 half_step * m.conductivity / (kVacuumPermittivity * m.relative_permittivity),
                 1.0f / m.relative_permeability,
                 half_step * m.magnetic_loss / (kVacuumPermeability * m.relative_permeability)};
}

} // namespace

// Shape::contains, src/scene.rs:60-81.
bool shape_contains(const dp_shape &s, const float p[3]) {
    if (s.kind == DP_SHAPE_BLOCK) {
        for (int a = 0; a < 3; ++a)
            if (!(std::fabs(p[a] - s.center[a]) <= 0.5f * s.size[a])) return false;
        return true;
    }
    if (s.kind == DP_SHAPE_SPHERE) {
        float d0 = p[0] - s.center[0], d1 = p[1] - s.center[1], d2 = p[2] - s.center[2];
        float r2 = d0 * d0;
        r2 += d1 * d1;
        r2 += d2 * d2;
        return r2 <= s.radius * s.radius;
    }
    return std::fabs(p[s.axis] - s.offset) <= 0.5f * s.thickness;
}

namespace {

// Cells a shape can possibly cover along one axis: the cells containing its
// two extremes, widened by two cells against rounding.  The exact membership
// test runs on every cell in the range, so this only skips cells whose
// centres lie well outside the shape (Shape::bounds, src/scene.rs:85-102).
void shape_range_impl(const ResolvedGrid &g, const dp_shape &s, int a, uint32_t &lo, uint32_t &hi) {
    float center = 0.0f, half = std::numeric_limits<float>::infinity();
    if (s.kind == DP_SHAPE_BLOCK) {
        center = s.center[a];
        half = 0.5f * std::fabs(s.size[a]);
    } else if (s.kind == DP_SHAPE_SPHERE) {
        center = s.center[a];
        half = std::fabs(s.radius);
    } else if (int(s.axis) == a) {
        center = s.offset;
        half = 0.5f * std::fabs(s.thickness);
    }
    lo = 0;
    hi = g.n[a] - 1;
    if (!std::isfinite(half) || !std::isfinite(center)) return;
    float c_lo = g.axes[a].coordinate(center - half), c_hi = g.axes[a].coordinate(center + half);
    long l = long(std::floor(c_lo)) - 2, h = long(std::floor(c_hi)) + 2;
    if (h < 0 || l > long(g.n[a]) - 1) {
        lo = 1;
        hi = 0; // empty
        return;
    }
    lo = uint32_t(std::max<long>(l, 0));
    hi = uint32_t(std::min<long>(h, long(g.n[a]) - 1));
}

} // namespace

void shape_cell_range(const ResolvedGrid &g, const dp_shape &s, int axis, uint32_t &lo, uint32_t &hi) {
    shape_range_impl(g, s, axis, lo, hi);
}

// Scene::material_indices, src/scene.rs:181-206: later shapes overwrite
// earlier ones, membership decided at the cell centre.
const std::vector<uint8_t> &Scene::material_index() const {
    if (indexed_) return index_cache_;
    const ResolvedGrid &g = grid;
    index_cache_.assign(g.cells() * index_bytes, 0);
    for (const dp_shape &sh : shapes) {
        uint32_t lo[3], hi[3];
        bool empty = false;
        for (int a = 0; a < 3; ++a) {
            shape_range_impl(g, sh, a, lo[a], hi[a]);
            if (lo[a] > hi[a]) empty = true;
        }
        if (empty) continue;
        const uint32_t material = sh.material;
        const long z0 = lo[2], z1 = hi[2];
#pragma omp parallel for schedule(dynamic, 1)
        for (long z = z0; z <= z1; ++z) {
            float p[3];
            p[2] = centers[axis_offset(2) + uint32_t(z)];
            for (uint32_t y = lo[1]; y <= hi[1]; ++y) {
                p[1] = centers[axis_offset(1) + y];
                const uint64_t row = (uint64_t(z) * g.n[1] + y) * g.n[0];
                for (uint32_t x = lo[0]; x <= hi[0]; ++x) {
                    p[0] = centers[x];
                    if (!shape_contains(sh, p)) continue;
                    uint8_t *cell = &index_cache_[(row + x) * index_bytes];
                    cell[0] = uint8_t(material);
                    if (index_bytes == 2) cell[1] = uint8_t(material >> 8);
                }
            }
        }
    }
    indexed_ = true;
    return index_cache_;
}

std::vector<float> Scene::cell_lookup(uint32_t samples) const {
    std::vector<float> lookup;
    lookup.reserve(3 * size_t(samples));
    for (int a = 0; a < 3; ++a) {
        const Axis1D &axis = grid.axes[a];
        const float length = axis.length();
        for (uint32_t k = 0; k < samples; ++k) {
            const float fraction = float(k) / float(samples - 1);
            lookup.push_back(axis.coordinate((fraction - 0.5f) * length));
        }
    }
    return lookup;
}

uint32_t Scene::lookup_samples() const {
    const uint32_t longest = std::max(std::max(grid.n[0], grid.n[1]), grid.n[2]);
    return std::min<uint32_t>(std::max<uint32_t>(4 * longest, 256), 8192);
}

Scene Scene::build(const dp_scene_desc &d) {
    Scene s;
    s.grid = ResolvedGrid::build(d.grid);
    s.grid.validate();
    s.boundary = d.boundary;
    if (d.material_count == 0 || d.materials == nullptr) invalid("a material table needs vacuum at index 0");
    if (d.material_count > 65536)
        throw Error(DP_ERR_UNSUPPORTED, "at most 65536 materials: the material index is stored as u16");
    if ((d.shape_count && !d.shapes) || (d.source_count && !d.sources)) invalid("null shape or source array");
    s.materials.assign(d.materials, d.materials + d.material_count);
    s.index_bytes = d.material_count <= 256 ? 1 : 2;
    s.shapes.assign(d.shapes, d.shapes + d.shape_count);
    s.sources.assign(d.sources, d.sources + d.source_count);
    for (const auto &sh : s.shapes)
        if (sh.material >= d.material_count) invalid("a shape refers to a material outside the table");
    for (const auto &src : s.sources) {
        if (src.polarization > 2 || src.axis > 2) invalid("an axis index must be 0, 1 or 2");
        if (src.shape > DP_SOURCE_PLANE_WAVE_BOX || src.waveform.kind > DP_WAVE_CONTINUOUS) invalid("unknown source or waveform kind");
        if (src.shape == DP_SOURCE_PLANE_WAVE_BOX) {
            if (src.polarization == src.axis) invalid("a plane wave's polarization must be transverse to its travel");
            uint32_t lo[3], hi[3];
            s.box_bounds(src, lo, hi);
            for (int a = 0; a < 3; ++a)
                if (!(lo[a] >= 1 && lo[a] < hi[a] && hi[a] + 2 <= s.grid.n[a]))
                    invalid("a total-field box needs a cell of scattered field and a wall cell beyond each face");
        }
    }

    const ResolvedGrid &g = s.grid;
    s.dt = g.time_step();

    // Grid::magnetic_gains / electric_gains, src/grid.rs:602-613.
    const float travel = kSpeedOfLight * s.dt;
    for (int a = 0; a < 3; ++a) {
        for (float w : g.axes[a].primary) s.magnetic_gains.push_back(travel / w);
        for (float w : g.axes[a].dual) s.electric_gains.push_back(travel / w);
        for (uint32_t i = 0; i < g.n[a]; ++i) s.centers.push_back(g.axes[a].position(float(i) + 0.5f));
        s.primary.insert(s.primary.end(), g.axes[a].primary.begin(), g.axes[a].primary.end());
        s.dual.insert(s.dual.end(), g.axes[a].dual.begin(), g.axes[a].dual.end());
    }

    // MaterialTable::coefficients, src/material.rs:207-212.
    for (const auto &m : s.materials) s.coefficients.push_back(material_coefficients(m, s.dt));

    // AbsorbingProfile::new, src/boundary.rs:100-145.
    const uint32_t span = g.n[0] + g.n[1] + g.n[2];
    s.absorber.assign(2 * size_t(span), 0.0f);
    uint32_t thickness = d.boundary.kind == DP_BOUNDARY_ABSORBING ? d.boundary.thickness : 0;
    if (d.boundary.kind != DP_BOUNDARY_PEC && d.boundary.kind != DP_BOUNDARY_ABSORBING) invalid("unknown boundary kind");
    if (thickness > 0) {
        for (int a = 0; a < 3; ++a)
            if (!(2 * size_t(thickness) < g.n[a])) invalid("absorbing layers do not fit in the axis");
        float target = d.boundary.target_reflection;
        if (!(target > 0.0f && target < 1.0f)) invalid("target reflection must lie in (0, 1)");
        const float order = 3.0f;
        const float t = float(thickness);
        const float peak = -(order + 1.0f) * std::log(target) * g.courant / (4.0f * t);
        for (int a = 0; a < 3; ++a) {
            const float outer = float(g.n[a] - 1);
            for (uint32_t i = 0; i < g.n[a]; ++i) {
                for (int h = 0; h < 2; ++h) {
                    float position = h ? float(i) + 0.5f : float(i);
                    float depth = std::fmax((t - position) / t, (t - (outer - position)) / t);
                    depth = depth < 0.0f ? 0.0f : (depth > 1.0f ? 1.0f : depth);
                    s.absorber[size_t(h) * span + s.axis_offset(a) + i] = peak * std::pow(depth, order);
                }
            }
        }
    }
    for (float v : s.absorber) s.absorber_peak = std::fmax(s.absorber_peak, v);

    // is_reversible, src/cpu.rs:209-215.
    s.reversible = s.absorber_peak == 0.0f;
    for (const Coeff &c : s.coefficients)
        if (!(c.electric_loss == 0.0f && c.magnetic_loss == 0.0f)) s.reversible = false;

    // Sheet apodization planes (src/source.rs:304-333 with the weight of
    // src/source.rs:441-455), evaluated once per sheet.
    s.source_weight.assign(s.sources.size(), -1);
    std::vector<StepInjection> probe;
    std::vector<BoxCorrections<float>> no_boxes(s.sources.size()); // boxes add no slots here
    std::vector<float> no_profiles;
    for (size_t k = 0, slot = 0; k < s.sources.size(); ++k) {
        const dp_source &src = s.sources[k];
        const size_t first = slot;
        slot += src.shape == DP_SOURCE_PLANE_WAVE_BOX ? 0 : 2;
        if (src.shape != DP_SOURCE_SHEET) continue;
        s.injections_in<float>(0.0f, probe, &no_boxes, &no_profiles); // the sheet's box does not depend on time
        const StepInjection &inj = probe[first];
        s.source_weight[k] = int32_t(s.weights.size());
        for (uint32_t dz = 0; dz < inj.extent[2]; ++dz)
            for (uint32_t dy = 0; dy < inj.extent[1]; ++dy)
                for (uint32_t dx = 0; dx < inj.extent[0]; ++dx) {
                    uint32_t coord[3] = {inj.origin[0] + dx, inj.origin[1] + dy, inj.origin[2] + dz};
                    float position[3];
                    g.cell_center(coord, position);
                    s.weights.push_back(injection_weight(inj, position));
                }
    }
    return s;
}

size_t Scene::injection_slots() const {
    size_t n = 0;
    for (const dp_source &src : sources) n += src.shape == DP_SOURCE_PLANE_WAVE_BOX ? 8 : 2;
    return n;
}

bool Scene::has_boxes() const {
    for (const dp_source &src : sources)
        if (src.shape == DP_SOURCE_PLANE_WAVE_BOX) return true;
    return false;
}

void Scene::box_bounds(const dp_source &src, uint32_t lo[3], uint32_t hi[3]) const {
    grid.cell_containing(src.box_low, lo);
    grid.cell_containing(src.box_high, hi);
}

// Source::injections, src/source.rs:280-403: two slots per source.
template <typename T>
void Scene::injections_in(T time, std::vector<InjectionOf<T>> &out, const std::vector<BoxCorrections<T>> *boxes,
                          std::vector<T> *profiles) const {
    out.clear();
    if (profiles) profiles->clear();
    const ResolvedGrid &g = grid;
    for (size_t k = 0; k < sources.size(); ++k) {
        const dp_source &src = sources[k];
        if (src.shape == DP_SOURCE_PLANE_WAVE_BOX) {
            if (!boxes || !profiles)
                throw Error(DP_ERR_UNSUPPORTED, "a total-field box's corrections depend on its incident line's history");
            const BoxCorrections<T> &b = (*boxes)[k];
            const int32_t base = int32_t(profiles->size());
            for (InjectionOf<T> inj : b.items) {
                if (inj.profile_offset >= 0) inj.profile_offset += base;
                out.push_back(inj);
            }
            profiles->insert(profiles->end(), b.profiles.begin(), b.profiles.end());
            continue;
        }
        const T value = T(src.amplitude) * waveform_in<T>(src.waveform, time);
        InjectionOf<T> a{}, b{};
        a.weight_offset = b.weight_offset = -1;
        a.component = b.component = src.polarization;
        if (src.shape == DP_SOURCE_POINT) {
            float position[3];
            for (int i = 0; i < 3; ++i) position[i] = src.at[i] + src.velocity[i] * static_cast<float>(time);
            g.cell_containing(position, a.origin);
            a.extent[0] = a.extent[1] = a.extent[2] = 1;
            // A mover outside the domain is silent, not clamped.
            a.value = g.contains(position) ? value : T(0);
            b = a;
            b.value = T(0);
        } else if (src.shape == DP_SOURCE_SHEET) {
            const int axis = int(src.axis);
            float position[3] = {0.0f, 0.0f, 0.0f};
            position[axis] = src.offset;
            uint32_t cell[3];
            g.cell_containing(position, cell);
            for (int i = 0; i < 3; ++i) {
                a.origin[i] = 0;
                a.extent[i] = g.n[i];
            }
            a.origin[axis] = cell[axis];
            a.extent[axis] = 1;
            a.inverse_waist_squared = 1.0f / (src.waist * src.waist);
            a.weight_offset = source_weight.empty() ? -1 : source_weight[k];
            a.value = value;
            b = a;
            b.value = T(0);
        } else {
            // Total-field / scattered-field plane, src/source.rs:334-401.
            const int travel = int(src.axis);
            float position[3] = {0.0f, 0.0f, 0.0f};
            position[travel] = src.offset;
            uint32_t cell[3];
            g.cell_containing(position, cell);
            const uint32_t plane = std::max<uint32_t>(cell[travel], 1);
            const float spacing = g.axes[travel].finest();
            const T dt_local = T(g.time_step());
            const T gain = T(kSpeedOfLight * g.time_step() / spacing);
            const T omega = T(2) * pi_in<T>() * T(src.waveform.frequency);
            const T half_k_spacing = std::asin(std::sin(T(0.5) * omega * dt_local) / gain);
            const T retard = half_k_spacing / omega;
            const int pol = int(src.polarization);
            const uint32_t h_axis = uint32_t(3 - travel - pol);
            const T h_sign = ((pol + 1) % 3) == travel ? T(-1) : T(1);
            for (int i = 0; i < 3; ++i) {
                a.extent[i] = b.extent[i] = g.n[i];
            }
            a.origin[travel] = plane;
            a.extent[travel] = 1;
            b.origin[travel] = plane - 1;
            b.extent[travel] = 1;
            a.value = gain * (T(src.amplitude) * waveform_in<T>(src.waveform, time - T(0.5) * dt_local + retard));
            b.component = h_axis;
            b.magnetic = 1;
            b.value = h_sign * gain * (T(src.amplitude) * waveform_in<T>(src.waveform, time - dt_local));
        }
        out.push_back(a);
        out.push_back(b);
    }
}

template void Scene::injections_in<float>(float, std::vector<InjectionOf<float>> &,
                                         const std::vector<BoxCorrections<float>> *, std::vector<float> *) const;
template void Scene::injections_in<double>(double, std::vector<InjectionOf<double>> &,
                                          const std::vector<BoxCorrections<double>> *, std::vector<double> *) const;

// ---------------------------------------------------------------------------
// Total-field boxes: the incident lines and the face corrections.
//
// Every E and H node of the Yee cell is inside the total field when its
// position lies within the box [lo, hi] (cell units, E-node indices): along
// its own axis an E node sits half a cell up and an H node on the index, so
// E_q is inside for lo_q <= i_q <= hi_q - 1 and H_q for lo_q <= i_q <= hi_q,
// and the other way round across.  An update that reads a node on the other
// side of the surface reads the wrong field there; it is corrected by the
// update's coefficient times the incident value at that node: added for a
// total node reading a scattered one, subtracted the other way.  With the
// incident E along p and H along h (a the travel axis) that leaves E_p and H_h
// on the two faces across a (uniform over the face), and the travel
// components on the side faces: H_a on the faces across h, E_a on the faces
// across p, whose incident values vary along a.  For the face across a at
// the entry this is exactly the reference's plane wave (src/source.rs:334-401).
// ---------------------------------------------------------------------------

namespace {
constexpr int kLineMargin = 8;  // line cells before the box and after it
constexpr int kLineTail = 64;   // absorbing cells at the line's far end
constexpr uint64_t kLineCheckpoint = 256;
float sign_if(bool b) { return b ? 1.0f : -1.0f; }
} // namespace

template <typename T> IncidentLines<T>::IncidentLines(const Scene &scene) {
    const ResolvedGrid &g = scene.grid;
    sources_ = scene.sources.size();
    dt_ = scene.dt;
    for (size_t k = 0; k < scene.sources.size(); ++k) {
        const dp_source &src = scene.sources[k];
        if (src.shape != DP_SOURCE_PLANE_WAVE_BOX) continue;
        Line l{};
        l.source = k;
        l.src = src;
        l.a = int(src.axis);
        l.p = int(src.polarization);
        l.h = 3 - l.a - l.p;
        uint32_t lo[3], hi[3];
        scene.box_bounds(src, lo, hi);
        for (int i = 0; i < 3; ++i) {
            l.lo[i] = int(lo[i]);
            l.hi[i] = int(hi[i]);
        }
        const int a = l.a, n_a = int(g.n[a]);
        l.first = l.lo[a] - kLineMargin;
        l.inject = kLineMargin / 2; // the line's own E row, lo_a - 4
        const int last = l.hi[a] + kLineMargin + kLineTail;
        const size_t count = size_t(last - l.first + 1);
        l.e.assign(count, T(0));
        l.hf.assign(count, T(0));
        l.ge.resize(count);
        l.gm.resize(count);
        l.le.assign(count, 0.0f);
        l.lm.assign(count, 0.0f);
        const uint32_t off_a = scene.axis_offset(a);
        for (size_t i = 0; i < count; ++i) {
            const int c = std::min(std::max(l.first + int(i), 0), n_a - 1);
            l.ge[i] = scene.electric_gains[off_a + uint32_t(c)];
            l.gm[i] = scene.magnetic_gains[off_a + uint32_t(c)];
        }
        // The tail: the absorbing profile's polynomial grading (the same form
        // as the grid's, src/boundary.rs:100-196) over the last cells.
        const float t = float(kLineTail);
        const float peak = -(3.0f + 1.0f) * std::log(1e-6f) * g.courant / (4.0f * t);
        const int tail0 = int(count) - kLineTail;
        for (int i = tail0; i < int(count); ++i) {
            const float de = std::fmin(float(i - tail0 + 1) / t, 1.0f);
            const float dh = std::fmin((float(i - tail0) + 1.5f) / t, 1.0f);
            l.le[size_t(i)] = peak * de * de * de;
            l.lm[size_t(i)] = peak * dh * dh * dh;
        }
        // The plane-wave drive of src/source.rs:334-401, for the line's row.
        const float spacing = g.axes[a].finest();
        const T dt = T(g.time_step());
        l.gain = T(kSpeedOfLight * g.time_step() / spacing);
        const T omega = T(2) * pi_in<T>() * T(src.waveform.frequency);
        const T half_k_spacing = std::asin(std::sin(T(0.5) * omega * dt) / l.gain);
        l.retard = half_k_spacing / omega;
        l.h_sign = ((l.p + 1) % 3) == a ? T(-1) : T(1);
        // Curl signs: E_p += sigma_e g (H_h[i] - H_h[i-1]); H_h -= sigma_h g
        // (E_p[i+1] - E_p[i]); H_a's term in E_p across h and E_a's in H_h
        // across p carry sigma_ha and sigma_ea.
        l.sigma_e = sign_if((l.p + 1) % 3 == a);
        l.sigma_h = sign_if((l.h + 1) % 3 == a);
        l.sigma_ha = sign_if((a + 2) % 3 == l.p);
        l.sigma_ea = sign_if((a + 2) % 3 == l.h);
        const uint32_t off_p = scene.axis_offset(l.p), off_h = scene.axis_offset(l.h);
        l.face_e[0] = scene.electric_gains[off_a + uint32_t(l.lo[a])];
        l.face_e[1] = scene.electric_gains[off_a + uint32_t(l.hi[a])];
        l.face_h[0] = scene.magnetic_gains[off_a + uint32_t(l.lo[a] - 1)];
        l.face_h[1] = scene.magnetic_gains[off_a + uint32_t(l.hi[a])];
        l.side_h[0] = scene.magnetic_gains[off_h + uint32_t(l.lo[l.h] - 1)];
        l.side_h[1] = scene.magnetic_gains[off_h + uint32_t(l.hi[l.h])];
        l.side_e[0] = scene.electric_gains[off_p + uint32_t(l.lo[l.p])];
        l.side_e[1] = scene.electric_gains[off_p + uint32_t(l.hi[l.p])];
        const int span = l.hi[a] - l.lo[a];
        profile_width_ += size_t(2 * (span + 1) + 2 * span);
        lines_.push_back(std::move(l));
    }
    std::vector<std::vector<T>> start;
    for (const Line &l : lines_) {
        start.push_back(l.e);
        start.push_back(l.hf);
    }
    checkpoints_.emplace_back(0, std::move(start));
}

template <typename T> const std::vector<BoxCorrections<T>> &IncidentLines<T>::at(uint64_t step) {
    if (cached_ == step) return cache_;
    if (state_ > step) {
        size_t c = checkpoints_.size() - 1;
        while (checkpoints_[c].first > step) --c;
        for (size_t i = 0; i < lines_.size(); ++i) {
            lines_[i].e = checkpoints_[c].second[2 * i];
            lines_[i].hf = checkpoints_[c].second[2 * i + 1];
        }
        state_ = checkpoints_[c].first;
    }
    while (state_ < step) advance(state_, nullptr);
    cache_.assign(sources_, BoxCorrections<T>{});
    advance(state_, &cache_);
    cached_ = step;
    return cache_;
}

// One step of every line (H, its drive, E, its drive), recording the box
// corrections of that step first when `out` is given.
template <typename T> void IncidentLines<T>::advance(uint64_t step, std::vector<BoxCorrections<T>> *out) {
    const T time = step_time<T>(step, dt_);
    const T dt = std::is_same_v<T, float> ? T(dt_) : T(double(dt_));
    for (Line &l : lines_) {
        const int a = l.a, p = l.p, h = l.h;
        const size_t count = l.e.size();
        auto E = [&](int cell) { return l.e[size_t(cell - l.first)]; };
        auto H = [&](int cell) { return l.hf[size_t(cell - l.first)]; };
        auto slot = [&](int component, bool magnetic) {
            InjectionOf<T> inj{};
            inj.component = uint32_t(component);
            inj.magnetic = magnetic ? 1u : 0u;
            inj.weight_offset = -1;
            inj.origin[a] = uint32_t(l.lo[a]);
            inj.extent[a] = uint32_t(l.hi[a] - l.lo[a]);
            inj.origin[p] = uint32_t(l.lo[p]);
            inj.extent[p] = uint32_t(l.hi[p] - l.lo[p]);
            inj.origin[h] = uint32_t(l.lo[h]);
            inj.extent[h] = uint32_t(l.hi[h] - l.lo[h] + 1);
            return inj;
        };
        BoxCorrections<T> *box = out ? &(*out)[l.source] : nullptr;
        std::vector<InjectionOf<T>> magnetic;
        if (box) {
            // H phase: the incident E at step·dt.
            for (int f = 0; f < 2; ++f) {
                InjectionOf<T> inj = slot(h, true);
                inj.origin[a] = uint32_t(f ? l.hi[a] : l.lo[a] - 1);
                inj.extent[a] = 1;
                inj.value = T(l.sigma_h * (f ? -l.face_h[1] : l.face_h[0])) * E(f ? l.hi[a] : l.lo[a]);
                magnetic.push_back(inj);
            }
            for (int f = 0; f < 2; ++f) {
                InjectionOf<T> inj = slot(a, true);
                inj.extent[a] = uint32_t(l.hi[a] - l.lo[a] + 1);
                inj.origin[h] = uint32_t(f ? l.hi[h] : l.lo[h] - 1);
                inj.extent[h] = 1;
                inj.value = T(1);
                inj.profile_offset = int32_t(box->profiles.size());
                inj.profile_axis = uint32_t(a);
                const T coef = T(l.sigma_ha * (f ? -l.side_h[1] : l.side_h[0]));
                for (int c = l.lo[a]; c <= l.hi[a]; ++c) box->profiles.push_back(coef * E(c));
                magnetic.push_back(inj);
            }
        }
        // H of the line: the same update the grid makes on a wave uniform
        // across it, and the absorbing tail.
        for (size_t i = 0; i < count; ++i) {
            const T next = i + 1 < count ? l.e[i + 1] : T(0);
            const T curl = T(l.sigma_h) * (T(l.gm[i]) * (next - l.e[i]));
            const T loss = T(l.lm[i]);
            l.hf[i] = loss == T(0) ? l.hf[i] - curl : ((T(1) - loss) * l.hf[i] - curl) / (T(1) + loss);
        }
        const T amplitude = T(l.src.amplitude);
        l.hf[size_t(l.inject - 1)] += l.h_sign * l.gain * (amplitude * waveform_in<T>(l.src.waveform, time - dt));
        if (box) {
            // E phase: the incident H at (step + 1/2)·dt.
            for (int f = 0; f < 2; ++f) {
                InjectionOf<T> inj = slot(p, false);
                inj.origin[a] = uint32_t(f ? l.hi[a] : l.lo[a]);
                inj.extent[a] = 1;
                inj.value = T(l.sigma_e * (f ? l.face_e[1] : -l.face_e[0])) * H(f ? l.hi[a] : l.lo[a] - 1);
                box->items.push_back(inj);
            }
            for (int f = 0; f < 2; ++f) {
                InjectionOf<T> inj = slot(a, false);
                inj.origin[p] = uint32_t(f ? l.hi[p] : l.lo[p]);
                inj.extent[p] = 1;
                inj.value = T(1);
                inj.profile_offset = int32_t(box->profiles.size());
                inj.profile_axis = uint32_t(a);
                const T coef = T(l.sigma_ea * (f ? l.side_e[1] : -l.side_e[0]));
                for (int c = l.lo[a]; c < l.hi[a]; ++c) box->profiles.push_back(coef * H(c));
                box->items.push_back(inj);
            }
            box->items.insert(box->items.end(), magnetic.begin(), magnetic.end());
        }
        for (size_t i = 1; i < count; ++i) {
            const T curl = T(l.sigma_e) * (T(l.ge[i]) * (l.hf[i] - l.hf[i - 1]));
            const T loss = T(l.le[i]);
            l.e[i] = loss == T(0) ? l.e[i] + curl : ((T(1) - loss) * l.e[i] + curl) / (T(1) + loss);
        }
        l.e[size_t(l.inject)] +=
            l.gain * (amplitude * waveform_in<T>(l.src.waveform, time - T(0.5) * dt + l.retard));
    }
    ++state_;
    if (state_ % kLineCheckpoint == 0 && checkpoints_.back().first < state_) {
        std::vector<std::vector<T>> snap;
        for (const Line &l : lines_) {
            snap.push_back(l.e);
            snap.push_back(l.hf);
        }
        checkpoints_.emplace_back(state_, std::move(snap));
    }
}

template class IncidentLines<float>;
template class IncidentLines<double>;

} // namespace diaphane
