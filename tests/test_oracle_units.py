"""The reference's unit known-answer tests, run against the oracle.

The reference ships no golden vectors and its Rust toolchain is not available,
so these — restated from the unit tests in src/grid.rs, src/material.rs,
src/boundary.rs, src/source.rs, src/cpu.rs, src/scene.rs (its rasterization
known answers) and src/timeline.rs — are what pin
the oracle's restatement of the reference's algorithm.  Each test names the
reference test it restates.
"""
import math

import numpy as np
import pytest

import oracle
from diaphane_gb300 import (Axis, Boundary, Extent, Grid, Material, MaterialTable, Scene, Shape, Source, Timeline,
                            Waveform, _abi)

C0 = 299792458.0
f32 = np.float32


def oracle_sim(scene, threads=8):
    return oracle.OracleSimulation(scene, threads=threads)


# ---- src/grid.rs:1014-1175 ---------------------------------------------------------

def test_axis_cycles():
    for axis in Axis:
        assert axis.next().next().next() == axis
        assert axis.prev() == axis.next().next()
        assert axis.next() != axis


def test_indexing_matches_strides():
    extent = Extent(5, 7, 11)
    strides = [1, 5, 35]
    for axis in range(3):
        coord = [1, 2, 3]
        base = extent.index(coord)
        coord[axis] += 1
        assert extent.index(coord) == base + strides[axis]


def test_time_step_respects_courant():
    info = oracle.grid_resolve(Grid.new(Extent.cube(16), 1e-3))
    expected = 0.5 * 1e-3 / C0
    assert abs(info["time_step"] - expected) < 1e-16


def test_rejects_unstable_courant():
    scene = Scene.empty(Extent.cube(16), 1e-3)
    scene.grid.courant = 0.9
    with pytest.raises(oracle.OracleError, match="Courant"):
        oracle_sim(scene)


def test_physical_coordinates_are_centred_and_round_trip():
    grid = Grid.new(Extent(40, 60, 80), 1e-3)
    size = oracle.grid_resolve(grid)["size"]
    assert all(abs(a - b) < 1e-7 for a, b in zip(size, (0.04, 0.06, 0.08)))
    assert oracle.grid_map(grid, 0, (0.0, 0.0, 0.0)) == (20.0, 30.0, 40.0)
    assert oracle.grid_map(grid, 1, (20.0, 30.0, 40.0)) == (0.0, 0.0, 0.0)
    for position in [(0.0, 0.0, 0.0), (0.011, -0.007, 0.03), (-0.02, 0.03, -0.04)]:
        p = tuple(float(f32(v)) for v in position)
        back = oracle.grid_map(grid, 1, oracle.grid_map(grid, 0, p))
        assert all(abs(a - b) < 1e-7 for a, b in zip(back, p))


def test_geometry_does_not_move_when_the_resolution_changes():
    size = (0.04, 0.06, 0.08)
    coarse, fine = Grid.for_size(size, 1000.0), Grid.for_size(size, 2000.0)
    assert oracle.grid_resolve(coarse)["extent"] == (40, 60, 80)
    assert oracle.grid_resolve(fine)["extent"] == (80, 120, 160)
    position = tuple(float(f32(v)) for v in (0.012, -0.018, 0.031))
    a, b = oracle.grid_map(coarse, 0, position), oracle.grid_map(fine, 0, position)
    assert all(abs(y - 2.0 * x) < 1e-3 for x, y in zip(a, b))


def test_a_cell_centre_lands_back_in_its_own_cell():
    grid = Grid.new(Extent(12, 14, 16), 1e-3)
    for coord in [(0, 0, 0), (4, 5, 6), (11, 13, 15), (6, 7, 8)]:
        centre = oracle.grid_map(grid, 3, coord)
        assert oracle.grid_map(grid, 2, centre) == tuple(float(c) for c in coord)
    assert oracle.grid_map(grid, 2, (-9.9, 0.0, 0.0)) == (0.0, 7.0, 8.0)
    assert oracle.grid_map(grid, 2, (9.9, 9.9, 9.9)) == (11.0, 13.0, 15.0)


def test_cell_centres_are_half_a_cell_in_from_the_corner():
    grid = Grid.new(Extent.cube(10), 1e-3)
    low, high = oracle.grid_map(grid, 3, (0, 0, 0)), oracle.grid_map(grid, 3, (9, 9, 9))
    assert all(abs(v + 0.0045) < 1e-7 for v in low)
    assert all(abs(v - 0.0045) < 1e-7 for v in high)


def test_dispersion_is_slower_along_axes_than_diagonals():
    axial = oracle.numerical_phase_velocity(0.5, 20.0, (1, 0, 0))
    diagonal = oracle.numerical_phase_velocity(0.5, 20.0, (1, 1, 1))
    assert axial < diagonal
    assert 0.99 < axial < 1.0
    assert 0.999 < diagonal <= 1.0
    fine = oracle.numerical_phase_velocity(0.5, 40.0, (1, 0, 0))
    assert 1.0 - fine < 1.0 - axial


# ---- src/material.rs:231-312 --------------------------------------------------------

def coefficient_table(materials, extent=16):
    scene = Scene.empty(Extent.cube(extent), 1e-3).with_boundary(Boundary.PEC)
    for m in materials:
        scene.materials.push(m)
    sim = oracle_sim(scene)
    return sim.table(_abi.DP_TABLE_COEFFICIENTS).reshape(-1, 4), sim


def test_vacuum_is_lossless_and_symmetric():
    table, sim = coefficient_table([])
    eg, el, mg, ml = table[0]
    assert el == 0.0 and ml == 0.0 and eg == mg == 1.0
    for which in (_abi.DP_TABLE_ELECTRIC_GAINS, _abi.DP_TABLE_MAGNETIC_GAINS):
        assert np.all(np.abs(sim.table(which) - 0.5) < 1e-6)


def test_perfect_conductor_pins_the_field_to_zero():
    table, _ = coefficient_table([Material.PERFECT_CONDUCTOR])
    eg, el, _, _ = (f32(v) for v in table[1])
    for e, curl in ((1.0, 5.0), (-3.0, -2.0)):
        assert ((f32(1.0) - el) * f32(e) + eg * f32(curl)) / (f32(1.0) + el) == 0.0


def test_matched_loss_has_equal_electric_and_magnetic_rates():
    for permittivity in (1.0, 2.25, 12.0):
        table, _ = coefficient_table([Material.matched_lossy(permittivity, 0.05)])
        _, el, _, ml = table[1]
        assert abs(el - ml) / el < 1e-5


def test_conductivity_raises_loss_without_touching_gain():
    table, _ = coefficient_table([Material.dielectric(4.0), Material.matched_lossy(4.0, 0.02)])
    assert table[1][0] == table[2][0]
    assert table[1][1] == 0.0 and table[2][1] > 0.0


def test_table_starts_with_vacuum_and_merges_duplicates():
    table = MaterialTable()
    assert table.get(MaterialTable.VACUUM) == Material.VACUUM
    glass = table.push(Material.refractive(1.5))
    assert glass == 1
    assert table.push(Material.refractive(1.5)) == glass
    assert table.push(Material.VACUUM) == MaterialTable.VACUUM
    assert len(table) == 2
    assert abs(table.peak_refractive_index() - 1.5) < 1e-6
    pec = MaterialTable()
    pec.push(Material.PERFECT_CONDUCTOR)
    assert pec.peak_refractive_index() == 1.0


# ---- src/boundary.rs:224-344 --------------------------------------------------------

def absorber(boundary=Boundary.DEFAULT, extent=Extent(40, 44, 48)):
    scene = Scene.empty(extent, 1e-3).with_boundary(boundary)
    sim = oracle_sim(scene)
    packed = sim.table(_abi.DP_TABLE_ABSORBER)
    n = extent.as_array()
    span = sum(n)
    offsets = [0, n[0], n[0] + n[1]]
    integer = [packed[offsets[a]:offsets[a] + n[a]] for a in range(3)]
    half = [packed[span + offsets[a]:span + offsets[a] + n[a]] for a in range(3)]

    def electric(axis, coord):  # electric_row: half along the component's own axis
        pick = lambda t: half[t] if t == axis else integer[t]
        return f32(pick(0)[coord[0]]) + (f32(pick(1)[coord[1]]) + f32(pick(2)[coord[2]]))

    def magnetic(axis, coord):
        pick = lambda t: integer[t] if t == axis else half[t]
        return f32(pick(0)[coord[0]]) + (f32(pick(1)[coord[1]]) + f32(pick(2)[coord[2]]))

    return sim, electric, magnetic, packed


def test_pec_has_no_loss_anywhere():
    sim, electric, magnetic, _ = absorber(Boundary.PEC)
    assert sim.absorber_peak() == 0.0
    assert electric(0, (0, 0, 0)) == 0.0 and magnetic(2, (39, 43, 47)) == 0.0


def test_interior_is_untouched_and_walls_are_damped():
    _, electric, magnetic, _ = absorber()
    assert electric(0, (20, 22, 24)) == 0.0 and magnetic(1, (20, 22, 24)) == 0.0
    corner, face = electric(0, (0, 0, 0)), electric(0, (0, 22, 24))
    assert corner > face > 0.0


def test_grading_is_monotone_into_the_wall():
    _, electric, _, _ = absorber()
    previous = math.inf
    for i in range(10):
        value = electric(1, (i, 22, 24))
        assert value <= previous
        previous = value
    assert electric(1, (12, 22, 24)) == 0.0


def test_both_walls_are_absorbing():
    _, _, magnetic, _ = absorber()
    assert magnetic(2, (20, 22, 0)) > 0.0 and magnetic(2, (20, 22, 47)) > 0.0


def test_peak_matches_the_closed_form():
    sim, _, _, _ = absorber()
    expected = -4.0 * math.log(1e-6) * 0.5 / 40.0
    assert abs(sim.absorber_peak() - expected) < 1e-5


def test_electric_and_magnetic_sample_different_positions():
    _, electric, magnetic, _ = absorber()
    assert electric(0, (3, 22, 24)) != magnetic(0, (3, 22, 24))


def test_packed_layout_has_integer_then_half_profiles():
    _, _, _, packed = absorber()
    assert packed.size == 2 * (40 + 44 + 48)


def test_rejects_a_layer_thicker_than_the_domain():
    with pytest.raises(oracle.OracleError, match="do not fit"):
        oracle_sim(Scene.empty(Extent.cube(12), 1e-3))


# ---- src/source.rs:458-652 ----------------------------------------------------------

def test_ricker_peaks_at_its_delay_and_is_zero_mean():
    w = Waveform.ricker(1e9)
    assert abs(oracle.waveform_evaluate(w, w.delay) - 1.0) < 1e-6
    assert abs(oracle.waveform_evaluate(w, 0.0)) < 1e-5
    steps, span = 20000, 4.0 * w.delay
    values = np.array([oracle.waveform_evaluate(w, float(f32(span) * f32(i) / f32(steps))) for i in range(steps)],
                      np.float32)
    assert abs(values.sum(dtype=np.float32) / steps) < 1e-4


def test_gaussian_pulse_envelope_has_the_requested_width():
    cycles = 10.0
    w = Waveform.gaussian_pulse(1e9, cycles)
    period = f32(1.0) / f32(1e9)

    def envelope(periods_from_peak):
        centre = f32(w.delay) + f32(periods_from_peak) * period
        return max(abs(oracle.waveform_evaluate(w, float(centre + (f32(i) / f32(256.0) - f32(0.5)) * period)))
                   for i in range(256))

    assert abs(envelope(0.0) - 1.0) < 0.02
    assert abs(envelope(0.5 * cycles) - 0.5) < 0.05   # FWHM: half the width out is half maximum
    assert envelope(2.0 * cycles) < 0.01
    assert abs(oracle.waveform_evaluate(w, 0.0)) < 1e-4


def test_continuous_wave_ramps_smoothly_from_rest():
    w = Waveform.continuous_wave(1e9, 3.0)
    assert oracle.waveform_evaluate(w, -1e-12) == 0.0 and oracle.waveform_evaluate(w, 0.0) == 0.0
    assert abs(oracle.waveform_evaluate(w, 0.25e-9)) < 0.15
    peak = max(abs(oracle.waveform_evaluate(w, 10e-9 + i * 1e-12)) for i in range(400))
    assert abs(peak - 1.0) < 0.01


def source_sim(source, extent=Extent(32, 40, 48)):
    return oracle_sim(Scene.empty(extent, 1e-3).with_boundary(Boundary.PEC).with_source(source))


def test_point_injection_covers_exactly_one_cell():
    sim = source_sim(Source.point((-11.5e-3, -14.5e-3, -17.5e-3), Axis.Z, Waveform.ricker(1e9)))
    inj = sim.injections(0.0)[0]
    assert tuple(inj.extent) == (1, 1, 1) and tuple(inj.origin) == (4, 5, 6) and inj.component == 2
    assert oracle.injection_weight(inj, (-11.5e-3, -14.5e-3, -17.5e-3)) == 1.0


def test_sheet_injection_spans_the_plane_and_apodizes_transversely():
    sim = source_sim(Source.sheet(Axis.X, -8e-3, 6e-3, Axis.Z, Waveform.ricker(1e9)))
    inj = sim.injections(0.0)[0]
    assert tuple(inj.origin) == (8, 0, 0) and tuple(inj.extent) == (1, 40, 48)
    assert abs(oracle.injection_weight(inj, (-8e-3, 0.0, 0.0)) - 1.0) < 1e-6
    assert abs(oracle.injection_weight(inj, (-8e-3, 6e-3, 0.0)) - math.exp(-1.0)) < 1e-6
    assert oracle.injection_weight(inj, (0.05, 0.0, 0.0)) == oracle.injection_weight(inj, (-8e-3, 0.0, 0.0))


def test_injection_value_follows_the_waveform():
    w = Waveform.ricker(1e9)
    sim = source_sim(Source.point((0.0, 0.0, 0.0), Axis.X, w).with_amplitude(3.0))
    assert abs(sim.injections(0.7e-9)[0].value - 3.0 * oracle.waveform_evaluate(w, 0.7e-9)) < 1e-6


def test_a_moving_point_tracks_its_velocity_and_goes_silent_when_it_leaves():
    w = Waveform.ricker(1e9)
    mover = source_sim(Source.point_moving((0.0, 0.0, 0.0), (1.5e8, 0.0, 0.0), Axis.Z, w))
    assert tuple(mover.injections(0.0)[0].origin) == (16, 20, 24)
    assert tuple(mover.injections(1e-10)[0].origin) == (31, 20, 24)
    assert mover.injections(w.delay)[0].value == 0.0
    sitter = source_sim(Source.point((0.0, 0.0, 0.0), Axis.Z, w))
    assert abs(sitter.injections(w.delay)[0].value) > 0.99


def test_a_plane_wave_makes_two_staggered_corrections():
    sim = source_sim(Source.plane_wave(Axis.X, 0.0, Axis.Z, Waveform.continuous_wave(1e9, 1.0)))
    electric, magnetic = sim.injections(10.13e-9)
    assert not electric.magnetic and magnetic.magnetic
    assert electric.component == 2 and magnetic.component == 1
    assert electric.origin[0] == magnetic.origin[0] + 1
    assert tuple(electric.extent) == (1, 40, 48) and tuple(magnetic.extent) == (1, 40, 48)
    assert electric.value > 0.0 and magnetic.value < 0.0


def test_sheet_clamps_a_position_past_the_far_wall():
    sim = source_sim(Source.sheet(Axis.Y, 9.9, 4e-3, Axis.X, Waveform.ricker(1e9)))
    assert sim.injections(0.0)[0].origin[1] == 39


# ---- src/cpu.rs:755-1036 -----------------------------------------------------------

def pulse_scene(extent):
    scene = Scene.empty(extent, 1e-3)
    frequency = scene.grid.frequency_for_resolution(20.0)
    return scene.with_source(Source.point((0.0, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))


def test_starts_at_rest():
    sim = oracle_sim(pulse_scene(Extent.cube(24)))
    assert sim.step_count() == 0 and sim.time() == 0.0 and sim.energy().total() == 0.0


def test_a_source_puts_energy_in_and_the_absorber_takes_it_out():
    sim = oracle_sim(pulse_scene(Extent.cube(48)))
    sim.advance_by(120)
    peak = sim.energy().total()
    assert peak > 0.0 and sim.is_finite()
    sim.advance_by(600)
    assert sim.energy().total() < peak * 1e-4


def mean_energy(sim, steps):
    total = 0.0
    for _ in range(steps):
        sim.advance()
        total += sim.energy().total()
    return total / steps


def test_a_pec_box_holds_on_to_its_energy():
    sim = oracle_sim(pulse_scene(Extent.cube(40)).with_boundary(Boundary.PEC))
    sim.advance_by(200)
    settled = mean_energy(sim, 200)
    sim.advance_by(2000)
    later = mean_energy(sim, 200)
    assert abs(later - settled) / settled < 1e-3


def test_the_two_energies_alternate_in_a_cavity():
    sim = oracle_sim(Scene.cavity(Extent.cube(40)))
    sim.advance_by(400)
    lo, hi = math.inf, -math.inf
    for _ in range(200):
        sim.advance()
        e = sim.energy()
        split = (e.electric - e.magnetic) / e.total()
        lo, hi = min(lo, split), max(hi, split)
    assert hi - lo > 0.3


def test_a_pulse_expands_at_about_the_speed_of_light():
    sim = oracle_sim(pulse_scene(Extent.cube(80)))
    radius, probe = 25, (65, 40, 40)
    arrival = None
    for step in range(1, 400):
        sim.advance()
        if abs(sim.sample_electric(Axis.Z, probe)) > 1e-4:
            arrival = step
            break
    assert arrival is not None
    travel = radius / 0.5
    assert travel * 0.9 < arrival < travel * 3.0


def test_a_perfect_conductor_expels_the_field():
    scene = pulse_scene(Extent.cube(40))
    metal = scene.materials.push(Material.PERFECT_CONDUCTOR)
    scene.shapes.append(Shape.block((10e-3, 0.0, 0.0), (8e-3, 20e-3, 20e-3), metal))
    sim = oracle_sim(scene)
    sim.advance_by(300)
    ez = sim.electric(Axis.Z).reshape(40, 40, 40)
    assert np.all(ez[10:30, 10:30, 26:34] == 0.0)


def test_stepping_back_undoes_stepping_forward():
    sim = oracle_sim(pulse_scene(Extent.cube(32)).with_boundary(Boundary.PEC))
    assert sim.is_reversible()
    sim.advance_by(60)
    before = np.concatenate([sim.read_electric(), sim.read_magnetic()])
    peak = np.abs(before).max()
    sim.advance_by(200)
    sim.reverse_by(200)
    assert sim.step_count() == 60
    after = np.concatenate([sim.read_electric(), sim.read_magnetic()])
    assert np.abs(before - after).max() < 1e-4 * peak


def test_reversing_all_the_way_returns_to_an_empty_domain():
    sim = oracle_sim(pulse_scene(Extent.cube(24)).with_boundary(Boundary.PEC))
    sim.advance_by(120)
    excited = sim.energy().total()
    sim.reverse_by(120)
    assert sim.step_count() == 0
    assert sim.energy().total() < excited * 1e-8


@pytest.mark.parametrize("with_conductor", [False, True])
def test_reversal_refuses_a_lossy_scene(with_conductor):
    scene = pulse_scene(Extent.cube(32))
    if with_conductor:
        scene = scene.with_boundary(Boundary.PEC)
        metal = scene.materials.push(Material.PERFECT_CONDUCTOR)
        scene.shapes.append(Shape.block((8e-3, 0.0, 0.0), (4e-3, 4e-3, 4e-3), metal))
    sim = oracle_sim(scene)
    assert not sim.is_reversible()
    sim.advance()
    with pytest.raises(oracle.OracleError, match="lossy"):
        sim.reverse()


def test_reset_returns_to_the_initial_state():
    sim = oracle_sim(pulse_scene(Extent.cube(24)))
    sim.advance_by(50)
    assert sim.energy().total() > 0.0
    sim.reset()
    assert sim.step_count() == 0 and sim.energy().total() == 0.0


def test_energy_density_sums_to_the_total_energy():
    sim = oracle_sim(pulse_scene(Extent.cube(24)))
    sim.advance_by(60)
    e = sim.read_electric().reshape(3, -1).astype(np.float32)
    h = sim.read_magnetic().reshape(3, -1).astype(np.float32)
    density = np.zeros(e.shape[1], np.float32)
    for a in range(3):
        density += f32(0.5) * (e[a] * e[a] + h[a] * h[a])
    widths = sim.table(_abi.DP_TABLE_PRIMARY)[:24]
    volume = float(np.float32(widths[0] * widths[0] * widths[0]))
    summed = float(np.sum(volume * density.astype(np.float64)))
    total = sim.energy().total()
    assert abs(summed - total) < total * 1e-4


# ---- src/scene.rs:511-568 (rasterization known answers) -----------------------------------
# Each checked on the oracle's index and on the product's host raster.

def index_tables(scene):
    from diaphane_gb300 import ResolvedScene
    ours = ResolvedScene(scene).table(_abi.DP_TABLE_MATERIAL_INDEX).astype(np.uint32)
    theirs = oracle_sim(scene).table(_abi.DP_TABLE_MATERIAL_INDEX)
    assert np.array_equal(ours, theirs)
    n = (scene.grid.extent.x, scene.grid.extent.y, scene.grid.extent.z)
    return lambda c: int(theirs[(c[2] * n[1] + c[1]) * n[0] + c[0]])


def test_an_empty_scene_is_all_vacuum():
    scene = Scene.empty(Extent.cube(24), 1e-3)
    at = index_tables(scene)
    assert all(at((x, y, z)) == MaterialTable.VACUUM for x in (0, 11, 23) for y in (0, 12, 23) for z in (0, 7, 23))


def test_shapes_rasterize_and_later_ones_win():
    # Conducting walls: the reference's raster needs no absorber, and a
    # 10-cell one does not fit the 16-cell domain (resolution would refuse it).
    scene = Scene.empty(Extent.cube(16), 1e-3).with_boundary(Boundary.PEC)
    glass = scene.materials.push(Material.refractive(1.5))
    metal = scene.materials.push(Material.PERFECT_CONDUCTOR)
    scene.shapes.append(Shape.block((0.0, 0.0, 0.0), (8e-3, 8e-3, 8e-3), glass))
    scene.shapes.append(Shape.sphere((0.0, 0.0, 0.0), 2e-3, metal))
    at = index_tables(scene)
    assert at((0, 0, 0)) == MaterialTable.VACUUM
    assert at((5, 5, 5)) == glass
    assert at((8, 8, 8)) == metal
    assert at((11, 11, 11)) == glass


def test_a_slab_spans_one_axis_only():
    scene = Scene.empty(Extent.cube(12), 1e-3).with_boundary(Boundary.PEC)
    glass = scene.materials.push(Material.refractive(2.0))
    scene.shapes.append(Shape.slab(Axis.Y, -1.5e-3, 3e-3, glass))
    at = index_tables(scene)
    assert at((0, 4, 11)) == glass
    assert at((11, 4, 0)) == glass
    assert at((5, 2, 5)) == MaterialTable.VACUUM
    assert at((5, 6, 5)) == MaterialTable.VACUUM


# ---- src/timeline.rs:215-423 (the Python Timeline over the oracle) ----------------------

def timeline_scene():
    return Scene.photon(Extent.cube(24))


def fingerprint(sim):
    return sim.read_electric()


def test_a_snapshot_restores_the_exact_state():
    sim = oracle_sim(timeline_scene())
    sim.advance_by(60)
    snap = sim.snapshot()
    expected = fingerprint(sim)
    sim.advance_by(40)
    assert not np.array_equal(fingerprint(sim), expected)
    sim.restore(snap)
    assert sim.step_count() == 60 and np.array_equal(fingerprint(sim), expected)
    assert snap.bytes() == 24 * 24 ** 3


def test_seeking_backwards_reproduces_the_forward_run_exactly():
    reference = oracle_sim(timeline_scene())
    reference.advance_by(90)
    sim = oracle_sim(timeline_scene())
    timeline = Timeline(25, 8)
    for _ in range(150):
        sim.advance_by(1)
        timeline.observe(sim)
    outcome = timeline.seek(sim, 90)
    assert sim.step_count() == 90
    assert np.array_equal(fingerprint(sim), fingerprint(reference))
    assert (outcome.kind, outcome.at, outcome.replayed) == ("keyframe", 75, 15)


def test_a_target_older_than_the_window_replays_from_the_start():
    sim = oracle_sim(timeline_scene())
    timeline = Timeline(20, 2)
    for _ in range(120):
        sim.advance_by(1)
        timeline.observe(sim)
    assert timeline.keyframe_count() == 2 and timeline.earliest() == 100
    reference = oracle_sim(timeline_scene())
    reference.advance_by(10)
    outcome = timeline.seek(sim, 10)
    assert (outcome.kind, outcome.replayed) == ("start", 10)
    assert np.array_equal(fingerprint(sim), fingerprint(reference))


def test_seeking_forward_just_steps_and_the_window_slides():
    sim = oracle_sim(timeline_scene())
    timeline = Timeline(10, 4)
    sim.advance_by(20)
    outcome = timeline.seek(sim, 35)
    assert (outcome.kind, outcome.replayed) == ("forward", 15) and sim.step_count() == 35
    assert timeline.seek(sim, 35).kind == "unchanged"
    sim = oracle_sim(timeline_scene())
    timeline = Timeline(10, 4)
    for _ in range(200):
        sim.advance_by(1)
        timeline.observe(sim)
    assert timeline.keyframe_count() == 4 and timeline.earliest() == 170
    assert timeline.bytes() == 4 * 24 * 24 ** 3


def test_batches_that_never_land_on_a_multiple_still_record():
    sim = oracle_sim(timeline_scene())
    timeline = Timeline(10, 8)
    sim.advance_by(10)
    timeline.observe(sim)
    timeline.observe(sim)
    assert timeline.keyframe_count() == 1
    sim = oracle_sim(timeline_scene())
    timeline = Timeline(10, 8)
    sim.advance_by(7)
    for _ in range(20):
        sim.advance_by(3)
        timeline.observe(sim)
    assert timeline.keyframe_count() >= 5


def test_recording_survives_a_seek_to_an_unaligned_step():
    sim = oracle_sim(timeline_scene())
    timeline = Timeline(10, 8)
    for _ in range(6):
        sim.advance_by(8)
        timeline.observe(sim)
    timeline.seek(sim, 13)
    before = timeline.keyframe_count()
    for _ in range(10):
        sim.advance_by(8)
        timeline.observe(sim)
    assert timeline.keyframe_count() > before
    assert timeline.seek(sim, 90).kind == "keyframe"


def test_scrubbing_a_lossless_scene_agrees_with_stepping_backwards():
    scene = Scene.cavity(Extent.cube(24)).with_boundary(Boundary.PEC)
    scrubbed = oracle_sim(scene)
    timeline = Timeline(20, 8)
    for _ in range(100):
        scrubbed.advance_by(1)
        timeline.observe(scrubbed)
    reversed_ = oracle_sim(scene)
    reversed_.advance_by(100)
    reversed_.reverse_by(30)
    timeline.seek(scrubbed, 70)
    assert scrubbed.step_count() == reversed_.step_count()
    a, b = fingerprint(scrubbed), fingerprint(reversed_)
    assert np.abs(a - b).max() < 1e-4 * np.abs(a).max()
