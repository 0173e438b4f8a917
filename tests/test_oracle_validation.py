"""The reference's analytic acceptance tests (tests/validation.rs and
tests/graded.rs), run against the oracle.

These compare against closed-form predictions of the *discrete* scheme and
against the reference's published measured figures (absorber -58 dB, grading
-32.5 / -52.4 dB, graded-vs-fine 0.6 %, graded cavity drift 4.9e-4).  Passing
them is the evidence that the oracle is a faithful restatement, since the
reference's Rust toolchain cannot run here.
"""
import math

import numpy as np
import pytest

import oracle
from diaphane_gb300 import Axis, Boundary, Extent, Grid, Material, Refinement, Scene, Shape, Source, Waveform

THREADS = 8


def sim_of(scene):
    return oracle.OracleSimulation(scene, threads=THREADS)


# ---- exact discrete plane wave (tests/validation.rs:28-240) --------------------------

class PlaneWave:
    def __init__(self, courant, direction, cells_per_wavelength, index):
        d = np.array(direction, np.float64)
        k = 2.0 * math.pi / cells_per_wavelength * d / np.linalg.norm(d)
        s = np.sin(0.5 * k)
        self.courant = courant
        self.wavenumber = k
        self.phase_rate = 2.0 * math.asin(courant * np.linalg.norm(s) / index)
        least = int(np.argmin(np.abs(s)))
        seed = np.zeros(3)
        seed[least] = 1.0
        e = np.cross(s, seed)
        self.electric_amplitude = e / np.linalg.norm(e)
        sigma = math.sin(0.5 * self.phase_rate)
        self.magnetic_amplitude = np.cross(s, self.electric_amplitude) * courant / sigma

    def phase_velocity(self):
        return self.phase_rate / (self.courant * np.linalg.norm(self.wavenumber))

    def free_space_cells(self):
        return 2.0 * math.pi * self.courant / self.phase_rate

    def fields(self, n, step):
        x, y, z = np.meshgrid(np.arange(n[0]), np.arange(n[1]), np.arange(n[2]), indexing="ij")
        dot = self.wavenumber[0] * x + self.wavenumber[1] * y + self.wavenumber[2] * z
        half_sum = 0.5 * self.wavenumber.sum()
        e = [self.electric_amplitude[a] * np.cos(self.phase_rate * step - (dot + 0.5 * self.wavenumber[a]))
             for a in range(3)]
        h = [self.magnetic_amplitude[a] *
             np.cos(self.phase_rate * (step - 0.5) - (dot + half_sum - 0.5 * self.wavenumber[a])) for a in range(3)]
        # x-major layout: transpose (x, y, z) arrays to z, y, x order before flattening
        flat = lambda arr: np.concatenate([c.transpose(2, 1, 0).ravel() for c in arr])
        return flat(e), flat(h)

    def seed(self, sim, n):
        e, h = self.fields(n, 0.0)
        sim.write_electric(e.astype(np.float32))
        sim.write_magnetic(h.astype(np.float32))

    def worst_error(self, sim, n, margin):
        e, h = self.fields(n, float(sim.step_count()))
        got_e, got_h = sim.read_electric().astype(np.float64), sim.read_magnetic().astype(np.float64)
        worst = 0.0
        for field, got in ((e, got_e), (h, got_h)):
            a = np.abs(field - got).reshape(3, n[2], n[1], n[0])
            worst = max(worst, float(a[:, margin:n[2] - margin, margin:n[1] - margin, margin:n[0] - margin].max()))
        return worst


def check_plane_wave(direction, cells, permittivity):
    side, steps = 96, 30
    scene = Scene.empty(Extent.cube(side), 1e-3).with_boundary(Boundary.PEC)
    if permittivity != 1.0:
        m = scene.materials.push(Material.dielectric(permittivity))
        scene.shapes.append(Shape.slab(Axis.X, 0.0, math.inf, m))
    wave = PlaneWave(0.5, direction, cells, math.sqrt(permittivity))
    sim = sim_of(scene)
    n = (side, side, side)
    wave.seed(sim, n)
    sim.advance_by(steps)
    error = wave.worst_error(sim, n, steps + 2)
    peak = max(np.abs(wave.magnetic_amplitude).max(), np.abs(wave.electric_amplitude).max())
    assert error < 1e-4 * peak, f"{direction} at {cells} cells/λ, εr={permittivity}: {error:e} of {peak:e}"
    return wave.phase_velocity()


@pytest.mark.parametrize("direction", [(1, 0, 0), (0, 0, 1), (1, 1, 1), (2, 1, 0)])
@pytest.mark.parametrize("cells", [10.0, 20.0])
def test_an_exact_plane_wave_propagates_exactly(direction, cells):
    check_plane_wave(direction, cells, 1.0)


def test_measured_phase_velocity_matches_the_dispersion_relation():
    for direction in [(1, 0, 0), (1, 1, 1), (2, 1, 0)]:
        for cells in (10.0, 20.0, 40.0):
            wave = PlaneWave(0.5, direction, cells, 1.0)
            measured = wave.phase_velocity()
            predicted = oracle.numerical_phase_velocity(0.5, float(np.float32(wave.free_space_cells())), direction)
            assert abs(measured - predicted) < 1e-4
            assert measured < 1.0


def test_dispersion_is_anisotropic_and_shrinks_with_refinement():
    velocity = lambda d, c: PlaneWave(0.5, d, c, 1.0).phase_velocity()
    axial, diagonal = velocity((1, 0, 0), 20.0), velocity((1, 1, 1), 20.0)
    assert axial < diagonal and 1.0 - axial < 0.005
    ratio = (1.0 - velocity((1, 0, 0), 10.0)) / (1.0 - velocity((1, 0, 0), 20.0))
    assert 3.5 < ratio < 4.5


@pytest.mark.parametrize("permittivity", [2.25, 4.0, 9.0])
def test_a_dielectric_slows_the_wave_by_its_refractive_index(permittivity):
    index = math.sqrt(permittivity)
    velocity = check_plane_wave((1, 0, 0), 20.0 * index, permittivity)
    assert abs(velocity - 1.0 / index) < 0.005 / index


def test_the_test_would_notice_a_wrong_dispersion_relation():
    scene = Scene.empty(Extent.cube(96), 1e-3).with_boundary(Boundary.PEC)
    wave = PlaneWave(0.5, (1, 0, 0), 10.0, 1.0)
    honest = wave.phase_rate
    wave.phase_rate = 0.5 * np.linalg.norm(wave.wavenumber)
    assert wave.phase_rate > honest
    sim = sim_of(scene)
    n = (96, 96, 96)
    wave.seed(sim, n)
    sim.advance_by(30)
    assert wave.worst_error(sim, n, 32) > 0.05


# ---- conservation, one-way injection, wall symmetry (tests/validation.rs:339-482) ----------

def mean_energy(sim, steps=200):
    total = 0.0
    for _ in range(steps):
        sim.advance()
        total += sim.energy().total()
    return total / steps


def test_a_closed_conducting_box_conserves_energy():
    sim = sim_of(Scene.cavity(Extent.cube(36)))
    sim.advance_by(400)
    early = mean_energy(sim)
    sim.advance_by(40_000)
    late = mean_energy(sim)
    assert sim.is_finite()
    assert abs(late - early) / early < 1e-3


def test_a_plane_wave_source_is_one_way():
    scene = Scene.empty(Extent(120, 32, 32), 1e-3)
    frequency = scene.grid.frequency_for_resolution(20.0)
    scene.sources.append(Source.plane_wave(Axis.X, -0.020, Axis.Z, Waveform.gaussian_pulse(frequency, 4.0)))
    sim = sim_of(scene)
    plane = 40
    total_peak = scattered_peak = 0.0
    for _ in range(900):
        sim.advance()
        ez = sim.electric(Axis.Z).reshape(32, 32, 120)[16, 16]
        scattered_peak = max(scattered_peak, float(np.abs(ez[12:plane - 10]).max()))
        total_peak = max(total_peak, float(np.abs(ez[plane + 10:108]).max()))
    assert 0.8 <= total_peak < 1.25
    leak = 20.0 * math.log10(scattered_peak / total_peak)
    assert leak < -25.0, f"leaks {leak:.1f} dB"


def test_a_conducting_box_cannot_tell_its_low_walls_from_its_high_ones():
    n = 24
    scene = Scene.empty(Extent.cube(n), 1e-3).with_boundary(Boundary.PEC)
    frequency = scene.grid.frequency_for_resolution(12.0)
    scene.sources.append(Source.point((0.0, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    sim = sim_of(scene)
    sim.advance_by(160)
    assert sim.is_finite()
    ez = sim.electric(Axis.Z).reshape(n, n, n)  # [z][y][x]
    peak = np.abs(ez).max()
    assert peak > 0.0
    assert np.all(ez[:, :, 0] == 0.0)
    mirrored = ez[:, :, ::-1][:, :, :n - 1]      # x -> n - x for x in 1..n
    worst = np.abs(ez[:, :, 1:] - mirrored).max()
    assert worst < 1e-6 * peak


# ---- absorbing layer reflection (tests/validation.rs:484-550) ----------------------------

def probe_trace(length, steps):
    scene = Scene.empty(Extent(length, 40, 40), 1e-3)
    frequency = scene.grid.frequency_for_resolution(20.0)
    position = oracle.grid_map(scene.grid, 1, (20.5, 20.0, 20.0))
    scene.sources.append(Source.point(position, Axis.Z, Waveform.ricker(frequency)))
    sim = sim_of(scene)
    trace = []
    for _ in range(steps):
        sim.advance()
        trace.append(sim.sample_electric(Axis.Z, (36, 20, 20)))
    return np.array(trace, np.float32)


def test_the_absorbing_layer_reflects_below_the_stated_level():
    near, reference = probe_trace(72, 380), probe_trace(200, 380)
    incident = float(np.abs(reference).max())
    reflected = float(np.abs(near - reference).max())
    decibels = 20.0 * math.log10(reflected / incident)
    assert decibels < -50.0
    # The reference reports about -58 dB for this measurement.
    assert -61.0 < decibels < -55.0, decibels


def test_a_propagating_packet_splits_its_energy_evenly():
    sim = sim_of(Scene.photon(Extent(80, 48, 48)))
    sim.advance_by(140)
    worst = 0.0
    for _ in range(60):
        sim.advance()
        e = sim.energy()
        worst = max(worst, abs(e.electric - e.magnetic) / e.total())
    assert worst < 0.1


# ---- graded grids (tests/graded.rs) ----------------------------------------------------

CELL, FINE = 1e-3, 0.25e-3
DOMAIN = (0.096, 0.040, 0.040)


def band(half_width, cell_size):
    return Refinement.across(Axis.X, 0.0, 2.0 * half_width, cell_size)


def test_stepping_back_survives_a_graded_grid():
    scene = Scene.cavity_on(Grid.graded((0.040, 0.028, 0.028), 1.0 / CELL, [band(0.004, FINE)]))
    sim = sim_of(scene)
    sim.advance_by(200)
    marked = sim.read_electric()
    excited = sim.energy().total()
    sim.advance_by(150)
    sim.reverse_by(150)
    returned = sim.read_electric()
    assert np.abs(marked - returned).max() < 1e-4 * np.abs(marked).max()
    sim.reverse_by(200)
    assert sim.energy().total() < 1e-8 * excited


def test_a_uniform_grid_is_a_spacing_whose_widths_are_equal():
    grid = Grid.new(Extent(40, 60, 80), CELL)
    scene = Scene.on_grid(grid).with_boundary(Boundary.PEC)
    sim = sim_of(scene)
    primary, dual = sim.table(6), sim.table(7)
    assert np.all(primary == np.float32(CELL)) and np.array_equal(primary, dual)
    assert np.all(sim.table(1) == np.float32(0.5))
    assert oracle.grid_resolve(grid)["worst_ratio"] == 1.0
    assert oracle.grid_map(grid, 0, (0.0, 0.0, 0.0)) == (20.0, 30.0, 40.0)


def test_grading_respects_the_growth_cap_and_the_walls():
    grid = Grid.graded(DOMAIN, 1.0 / CELL, [band(4e-3, FINE)])
    info = oracle.grid_resolve(grid)
    assert info["worst_ratio"] <= 1.15 + 1e-5
    assert all(abs(s - d) < 1e-6 for s, d in zip(info["size"], DOMAIN))
    assert info["finest"] < 1.2 * FINE and info["coarsest"] > 0.9 * CELL
    extent = info["extent"]
    for fraction in (0.0, 0.1, 0.5, 0.9):
        coord = tuple(int((e - 1) * fraction) for e in extent)
        centre = oracle.grid_map(grid, 3, coord)
        assert oracle.grid_map(grid, 2, centre) == tuple(float(c) for c in coord)


def test_grading_buys_cells_rather_than_accuracy():
    info = oracle.grid_resolve(Grid.graded(DOMAIN, 1.0 / CELL, [band(4e-3, FINE)]))
    saving = round(DOMAIN[0] / FINE) / info["extent"][0]
    assert saving > 2.5
    assert info["extent"][1] == info["extent"][2] == 40
    assert abs(info["finest"] / FINE - 1.0) < 0.05


def trace(grid, steps):
    scene = Scene.on_grid(grid)
    frequency = scene.grid.frequency_for_resolution(20.0)
    scene.sources.append(Source.point((-0.012, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    probe = tuple(int(v) for v in oracle.grid_map(grid, 2, (-0.004, 0.0, 0.0)))
    sim = sim_of(scene)
    out = []
    for _ in range(steps):
        sim.advance()
        out.append(sim.sample_electric(Axis.Z, probe))
    return np.array(out, np.float32), sim.time_step()


def uniformly_fine():
    return Grid.graded(DOMAIN, 1.0 / CELL, [Refinement.across(Axis.X, 0.0, 2.0 * DOMAIN[0], FINE)])


def resample(values, source_step, count, target_step):
    out = []
    for i in range(count):
        position = np.float32(i) * np.float32(target_step) / np.float32(source_step)
        low = int(np.floor(position))
        fraction = position - np.float32(low)
        at = lambda k: values[k] if k < len(values) else np.float32(0.0)
        out.append(at(low) * (np.float32(1.0) - fraction) + at(low + 1) * fraction)
    return np.array(out, np.float32)


def test_a_graded_grid_gives_the_same_answer_as_a_uniformly_fine_one():
    steps = 300
    measured, graded_step = trace(Grid.graded(DOMAIN, 1.0 / CELL, [band(0.02, FINE)]), steps)
    fine_step = oracle.grid_resolve(uniformly_fine())["time_step"]
    expected, _ = trace(uniformly_fine(), int(np.float32(steps) * np.float32(graded_step) / np.float32(fine_step)) + 2)
    expected = resample(expected, fine_step, len(measured), graded_step)
    peak = np.abs(expected).max()
    worst = np.abs(measured - expected).max()
    assert peak > 0.0 and worst < 0.06 * peak
    # The reference reports 0.6 % of peak for this comparison.
    assert worst / peak < 0.012, worst / peak


def grading_reflection(max_ratio):
    steps = 340
    measured, _ = trace(Grid.graded(DOMAIN, 1.0 / CELL, [band(0.014, FINE)], max_ratio), steps)
    reference, _ = trace(uniformly_fine(), steps)
    incident = np.abs(reference).max()
    return 20.0 * math.log10(np.abs(measured - reference).max() / incident)


def test_a_grading_transition_reflects_and_grading_gently_reflects_less():
    default, gentle = grading_reflection(1.15), grading_reflection(1.05)
    assert gentle < default - 3.0
    assert default < -30.0
    # The reference reports -32.5 dB at 1.15 and -52.4 dB at 1.05.
    assert abs(default - (-32.5)) < 1.5 and abs(gentle - (-52.4)) < 1.5, (default, gentle)


def test_a_graded_conducting_box_conserves_energy():
    sim = sim_of(Scene.cavity_on(Grid.graded((0.024,) * 3, 1000.0, [band(4e-3, 0.4e-3)])))
    sim.advance_by(400)
    early = mean_energy(sim)
    sim.advance_by(20_000)
    late = mean_energy(sim)
    assert sim.is_finite()
    drift = abs(late - early) / early
    # The reference asserts < 1e-3 (its documentation quotes 4.9e-4; the
    # oracle measures 2.4e-4 while reproducing the other published figures).
    assert drift < 1e-3


def test_the_documented_graded_drift_lies_within_the_spread_of_the_windowed_statistic():
    """Why the oracle's 2.4e-4 and the documented 4.9e-4 differ: the statistic
    compares two 200-step means of the instantaneous energy, which still
    beats with the cavity's modes, so where the late window sits moves the
    figure by several times.  Sliding the late window (steps 20,601-20,800 in
    tests/graded.rs:315-350) by up to 100 steps either way spans the
    documented value; a longer window settles an order of magnitude lower."""
    sim = sim_of(Scene.cavity_on(Grid.graded((0.024,) * 3, 1000.0, [band(4e-3, 0.4e-3)])))
    sim.advance_by(400)
    early = mean_energy(sim)
    sim.advance_by(20_000 - 100)
    energies = []
    for _ in range(400):
        sim.advance()
        energies.append(sim.energy().total())
    energies = np.array(energies)
    drifts = {offset: abs(energies[100 + offset:300 + offset].mean() - early) / early
              for offset in range(-100, 101, 25)}
    assert abs(drifts[0] - 2.4e-4) < 0.1e-4, drifts[0]  # the reference's own windows
    assert min(drifts.values()) < 4.9e-4 < max(drifts.values()), drifts
    assert max(drifts.values()) < 1e-3  # the asserted bound holds for every placement


# ---- total-field box (an extension; pinned by the one-way method above) ---------------

def box_scene(travel: Axis, polarization: Axis, n: int = 48, lo: int = 14, hi: int = 34) -> Scene:
    """A vacuum cube with a total-field box whose faces sit at cells lo and
    hi on every axis, a Gaussian pulse at 20 cells per wavelength."""
    scene = Scene.empty(Extent.cube(n), 1e-3)
    frequency = scene.grid.frequency_for_resolution(20.0)

    def metres(cell: int) -> float:
        return (cell + 0.5) * 1e-3 - n * 1e-3 / 2.0

    scene.sources.append(Source.plane_wave_box(travel, (metres(lo),) * 3, (metres(hi),) * 3, polarization,
                                               Waveform.gaussian_pulse(frequency, 4.0)))
    return scene


@pytest.mark.parametrize("travel,polarization", [(Axis.X, Axis.Z), (Axis.X, Axis.Y), (Axis.Y, Axis.X),
                                                 (Axis.Y, Axis.Z), (Axis.Z, Axis.X), (Axis.Z, Axis.Y)])
def test_a_total_field_box_keeps_its_wave_inside(travel, polarization):
    # The reference's one-way measurement (tests/validation.rs:375-429) over
    # every side of the box: the wave crosses the total field at full
    # strength while everything outside stays at roundoff, because the
    # incident line propagates exactly what the grid does, dispersion
    # included, and each face subtracts it where the stencil reaches across.
    n, lo, hi = 48, 14, 34
    sim = sim_of(box_scene(travel, polarization, n, lo, hi))
    inside = np.zeros((n, n, n), dtype=bool)
    inside[lo:hi + 1, lo:hi + 1, lo:hi + 1] = True
    total_peak = scattered_peak = 0.0
    for step in range(320):
        sim.advance()
        if step % 4:
            continue
        e = [sim.electric(a).reshape(n, n, n) for a in (Axis.X, Axis.Y, Axis.Z)]
        total_peak = max(total_peak, float(np.abs(e[int(polarization)][inside]).max()))
        scattered_peak = max(scattered_peak, max(float(np.abs(c[~inside]).max()) for c in e))
    assert 0.8 <= total_peak < 1.25, total_peak
    leak = 20.0 * math.log10(max(scattered_peak, 1e-30) / total_peak)
    assert leak < -80.0, f"the box leaks {leak:.1f} dB"
