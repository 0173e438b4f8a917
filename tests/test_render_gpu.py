"""The headless volume renderer against the oracle's restatement of the
reference shader (examples/common/shaders/volume.wgsl) and exposure control
(examples/common/render.rs).

The peak reduction is a max, so its eight slots must agree bit for bit.  The
images go through exp/log/pow, whose last-ulp results differ between CUDA and
numpy, so every channel must agree within one 8-bit step and nearly every
pixel exactly."""
import numpy as np
import pytest

import oracle
from oracle import render as ref
from diaphane_gb300 import Axis, Extent, Grid, Refinement, Scene, Simulation, _abi, workloads
from diaphane_gb300.render import Renderer, View, write_png
from tests import scenes

pytestmark = pytest.mark.gpu

WIDTH, HEIGHT = 96, 64


def lookup_of(scene, extent):
    """Grid::cell_lookup from the oracle's own coordinate map."""
    samples = min(max(4 * max(extent), 256), 8192)
    size = oracle.grid_resolve(scene.grid)["size"]
    lookup = np.empty(3 * samples, np.float32)
    for k in range(samples):
        fraction = np.float32(k) / np.float32(samples - 1)
        position = [(fraction - np.float32(0.5)) * np.float32(size[a]) for a in range(3)]
        cell = oracle.grid_map(scene.grid, _abi.DP_MAP_TO_CELL, position)
        for a in range(3):
            lookup[a * samples + k] = cell[a]
    box = [np.float32(size[a]) / np.float32(scene.grid.spec()[0].cell_size) for a in range(3)]
    return lookup, samples, box


def fields_of(sim):
    n = sim.cells
    return (sim.read_electric().reshape(3, n), sim.read_magnetic().reshape(3, n),
            sim.read_intensity() if sim.accumulated_steps() else np.zeros(n, np.float32))


def compare(got, want, name):
    diff = np.abs(got.astype(np.int16) - want.astype(np.int16))
    assert diff.max() <= 1, (name, int(diff.max()))
    assert (diff == 0).mean() > 0.99, (name, float((diff == 0).mean()))


def graded_cavity():
    grid = Grid.graded((0.040, 0.028, 0.028), 1000.0, [Refinement.across(Axis.X, 0.0, 0.008, 0.25e-3)])
    return Scene.cavity_on(grid)


SCENES = {"heterogeneous 48": lambda: (workloads.heterogeneous(48, spheres=6), 70),
          "graded cavity": lambda: (graded_cavity(), 90),
          "plane wave": lambda: (scenes.plane_wave()[0], 60)}


@pytest.mark.parametrize("name", sorted(SCENES))
def test_frames_match_the_oracle_in_every_view(name):
    scene, steps = SCENES[name]()
    sim = Simulation(scene)
    sim.set_accumulate_intensity(True)
    sim.advance_by(steps)
    lookup, samples, box = lookup_of(scene, sim.extent)
    renderer = Renderer(sim, WIDTH, HEIGHT)
    renderer.measure()
    state = ref.Exposure()
    e, h, intensity = fields_of(sim)
    slots = ref.measure_peak(e, h, intensity, sim.accumulated_steps())
    peaks, _, _ = renderer.state()
    assert np.array_equal(peaks.view(np.uint32), slots.view(np.uint32))
    for mode in range(8):
        view = View(mode=mode, yaw=0.9 + 0.3 * mode, scrub=mode % 2 == 0, played=0.6, window_start=0.25)
        renderer.draw(view, advanced=True)
        ref.update_scale(state, slots, True, mode)
        image = renderer.pixels()
        _, scale, comps = renderer.state()
        assert np.float32(scale) == np.float32(state.scale) and list(comps) == state.components, mode
        want = ref.render(e, h, intensity, sim.extent, lookup, samples, box, ref.View(**view.__dict__), state,
                          sim.accumulated_steps(), WIDTH, HEIGHT)
        compare(image, want, (name, mode))
        assert image[..., :3].std() > 1.0, "a blank frame"


def test_exposure_follows_the_field_a_frame_late(tmp_path):
    """The exposure folds in the previous frame's reduction, rising fast and
    falling slowly, and only when the solver advanced (render.rs:281-325);
    the frame also goes out as a PNG."""
    sim = Simulation(Scene.photon(Extent.cube(40)))
    renderer = Renderer(sim, 48, 32)
    state = ref.Exposure()
    renderer.measure()
    e, h, intensity = fields_of(sim)
    pending = ref.measure_peak(e, h, intensity, 0)
    scales = []
    for frame in range(12):
        sim.advance_by(10)
        advanced = frame != 5
        renderer.draw(View(), advanced=advanced)
        ref.update_scale(state, pending, advanced, _abi.DP_VIEW_FIELDS)
        e, h, intensity = fields_of(sim)
        pending = ref.measure_peak(e, h, intensity, 0)
        _, scale, comps = renderer.state()
        assert np.float32(scale) == np.float32(state.scale) and list(comps) == state.components, frame
        scales.append(scale)
    assert scales[5] == scales[4]  # a paused frame keeps its exposure
    assert scales[-1] > 0
    path = tmp_path / "frame.png"
    write_png(path, renderer.pixels())
    assert path.read_bytes()[:8] == b"\x89PNG\r\n\x1a\n"
