"""Edge shapes and limits of the GPU path, each against the oracle bit for bit:
the smallest grids the reference accepts (2 cells on an axis), rows shorter
than a lane's cells, odd extents, more sources than the fused step carries
(the handle falls back to the one-thread-per-cell passes), and a zero-step
advance."""
import numpy as np
import pytest

import oracle
from diaphane_gb300 import (DP_KERNEL_AUTO, DP_KERNEL_FUSED, DP_KERNEL_NAIVE, Axis, Batch, Boundary, DiaphaneError,
                            Extent, Material, ResolvedScene, Scene, Shape, Source, Waveform)
from diaphane_gb300 import Simulation, workloads
from diaphane_gb300._abi import DP_ERR_UNSUPPORTED

pytestmark = pytest.mark.gpu


def bits(a):
    return a.view(np.uint32)


def small_scene(extent, sources=1):
    scene = Scene.empty(Extent(*extent), 1e-3).with_boundary(Boundary.PEC)
    glass = scene.materials.push(Material.dielectric(2.5))
    scene.shapes.append(Shape.block((0.0, 0.0, 0.0), (2e-3, 2e-3, 2e-3), glass))
    frequency = scene.grid.frequency_for_resolution(8.0)
    for k in range(sources):
        at = [((k * 7 + 3 * a) % max(n, 1) - n / 2 + 0.5) * 1e-3 for a, n in enumerate(extent)]
        scene.sources.append(Source.point(at, Axis(k % 3), Waveform.ricker(frequency)))
    return scene


@pytest.mark.parametrize("extent", [(2, 2, 2), (3, 5, 7), (4, 2, 9), (5, 3, 2), (130, 3, 2), (33, 2, 40)])
@pytest.mark.parametrize("kernel", [DP_KERNEL_FUSED, DP_KERNEL_NAIVE])
def test_small_and_odd_grids_match_the_oracle(extent, kernel, threads):
    scene = small_scene(extent)
    ref = oracle.OracleSimulation(scene, threads=threads)
    sim = Simulation(scene, kernel=kernel)
    assert sim.kernel == kernel
    ref.advance_by(40)
    sim.advance_by(40)
    assert np.array_equal(bits(sim.read_electric()), bits(ref.read_electric())), extent
    assert np.array_equal(bits(sim.read_magnetic()), bits(ref.read_magnetic())), extent


def test_more_sources_than_the_fused_step_carries_fall_back_exactly(threads):
    scene = small_scene((24, 20, 18), sources=17)
    with pytest.raises(DiaphaneError) as err:
        Simulation(scene, kernel=DP_KERNEL_FUSED)
    assert err.value.status == DP_ERR_UNSUPPORTED
    sim = Simulation(scene, kernel=DP_KERNEL_AUTO)
    assert sim.kernel == DP_KERNEL_NAIVE
    ref = oracle.OracleSimulation(scene, threads=threads)
    sim.advance_by(60)
    ref.advance_by(60)
    assert np.array_equal(bits(sim.read_electric()), bits(ref.read_electric()))
    assert np.array_equal(bits(sim.read_magnetic()), bits(ref.read_magnetic()))


def test_a_zero_step_advance_changes_nothing():
    sim = Simulation(small_scene((16, 12, 10)))
    sim.advance_by(7)
    before = sim.read_electric()
    sim.advance_by(0)
    assert sim.step_count() == 7
    assert np.array_equal(bits(sim.read_electric()), bits(before))


def test_a_batch_refuses_a_scene_with_too_many_sources():
    batch = Batch(1 << 28, chunk_steps=4, max_scenes=2)
    with pytest.raises(DiaphaneError) as err:
        batch.add(ResolvedScene(small_scene((16, 12, 10), sources=5)), 10)
    assert err.value.status == DP_ERR_UNSUPPORTED


def test_past_256_materials_the_index_widens_and_stays_exact(threads):
    """The reference indexes materials with u32; past 256 this library keeps a
    u16 index, steps with the one-thread-per-cell passes (the fused step and
    the batch stage a u8 index) and matches the oracle bit for bit."""
    from tests.test_setup_parity import many_materials
    scene = many_materials(300, side=28)
    frequency = scene.grid.frequency_for_resolution(8.0)
    scene.sources.append(Source.point((0.0005, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    resolved = ResolvedScene(scene)
    assert resolved.index_bytes == 2
    with pytest.raises(DiaphaneError) as err:
        Simulation(resolved, kernel=DP_KERNEL_FUSED)
    assert err.value.status == DP_ERR_UNSUPPORTED
    with pytest.raises(DiaphaneError) as err:
        Batch(1 << 28, chunk_steps=4, max_scenes=2).add(resolved, 10)
    assert err.value.status == DP_ERR_UNSUPPORTED
    sim = Simulation(resolved)
    assert sim.kernel == DP_KERNEL_NAIVE
    ref = oracle.OracleSimulation(scene, threads=threads)
    sim.advance_by(60)
    ref.advance_by(60)
    assert np.array_equal(bits(sim.read_electric()), bits(ref.read_electric()))
    assert np.array_equal(bits(sim.read_magnetic()), bits(ref.read_magnetic()))
    e, m = sim.energy(), ref.energy()
    assert e.total() == pytest.approx(m.total(), rel=1e-9)


def test_energy_density_and_samples_match_the_oracle(threads):
    """cpu::Simulation::energy_density and sample_* (src/cpu.rs:154-161,
    689-703) on the device."""
    scene = workloads.mixed_scene(21, lo=30, hi=46)
    sim = Simulation(scene)
    sim.set_accumulate_intensity(True)
    ref = oracle.OracleSimulation(scene, threads=threads)
    ref.set_accumulate_intensity(True)
    sim.advance_by(70)
    ref.advance_by(70)
    assert np.array_equal(bits(sim.energy_density()), bits(ref.energy_density()))
    n = sim.extent
    for coord in [(0, 0, 0), (n[0] // 2, n[1] // 3, n[2] // 4), (n[0] - 1, n[1] - 1, n[2] - 1)]:
        for axis in (Axis.X, Axis.Y, Axis.Z):
            assert np.float32(sim.sample_electric(axis, coord)) == np.float32(ref.sample_electric(axis, coord))
            assert np.float32(sim.sample_magnetic(axis, coord)) == np.float32(ref.sample_magnetic(axis, coord))
    with pytest.raises(DiaphaneError):
        sim.sample_electric(Axis.X, (n[0], 0, 0))


def test_a_wait_that_gave_up_is_reported_once_and_the_handle_stays_usable(threads):
    """A fused step whose bounded ring wait runs out sets an error flag and
    returns; the next wait reports DP_ERR_TIMEOUT and clears it.  The flag is
    raised from the host here, so no wait on the GPU is made to run out."""
    import ctypes as C
    from diaphane_gb300 import _abi
    from diaphane_gb300._abi import DP_ERR_TIMEOUT
    fn = _abi.lib().dp_internal_raise_wait_error
    fn.restype, fn.argtypes = C.c_int, [C.c_void_p]
    scene = small_scene((24, 20, 16))
    sim = Simulation(scene, kernel=DP_KERNEL_FUSED)
    sim.advance_by(5)
    assert fn(sim.handle) == 0
    with pytest.raises(DiaphaneError) as err:
        sim.wait()
    assert err.value.status == DP_ERR_TIMEOUT
    sim.wait()  # reported once
    sim.advance_by(10)
    ref = oracle.OracleSimulation(scene, threads=threads)
    ref.advance_by(15)
    assert np.array_equal(bits(sim.read_electric()), bits(ref.read_electric()))


def test_a_ring_wait_that_runs_out_on_the_gpu_is_reported_and_the_run_recovers(threads):
    """The device half of the bounded wait (the reference's host timeout is
    src/gpu.rs:616-622): with the plane-wait budget set to zero every CTA of a
    fused step gives up at its first plane, sets the error flag, lets the
    loads it issued land (the drain keeps its full bound) and exits.  The
    host reports DP_ERR_TIMEOUT once; after the budget is restored and a
    snapshot restored, the run continues bit-identical to the oracle."""
    import ctypes as C
    from diaphane_gb300 import _abi
    from diaphane_gb300._abi import DP_ERR_TIMEOUT
    budget = _abi.lib().dp_internal_ring_wait_budget
    budget.restype, budget.argtypes = C.c_int, [C.c_void_p, C.c_longlong]
    scene = small_scene((40, 20, 16))
    sim = Simulation(scene, kernel=DP_KERNEL_FUSED)
    sim.advance_by(5)
    snapshot = sim.snapshot()
    assert budget(sim.handle, 0) == 0
    try:
        sim.advance_by(2)
        with pytest.raises(DiaphaneError) as err:
            sim.wait()
        assert err.value.status == DP_ERR_TIMEOUT
    finally:
        assert budget(sim.handle, -1) == 0
    sim.wait()  # reported once
    sim.restore(snapshot)
    sim.advance_by(10)
    ref = oracle.OracleSimulation(scene, threads=threads)
    ref.advance_by(15)
    assert np.array_equal(bits(sim.read_electric()), bits(ref.read_electric()))
    assert np.array_equal(bits(sim.read_magnetic()), bits(ref.read_magnetic()))


def test_autotuning_keeps_the_state_and_the_results(threads):
    """dp_sim_autotune times the fused step's plans from the current state and
    restores it exactly: the run continues bit-identical to the oracle."""
    from tests import scenes
    scene, _ = scenes.graded()
    sim = Simulation(scene, kernel=DP_KERNEL_FUSED)
    sim.set_accumulate_intensity(True)
    sim.advance_by(12)
    before_e, before_i = sim.read_electric(), sim.read_intensity()
    tuning = sim.autotune(steps=3)
    assert tuning["candidates"] >= 4 and tuning["ms_per_step"] > 0
    assert tuning["cells_per_lane"] in (1, 2, 4) and tuning["tile_y"] in (8, 16)
    assert sim.step_count() == 12 and sim.accumulated_steps() == 12
    assert np.array_equal(bits(sim.read_electric()), bits(before_e))
    assert np.array_equal(bits(sim.read_intensity()), bits(before_i))
    sim.advance_by(28)
    ref = oracle.OracleSimulation(scene, threads=threads)
    ref.set_accumulate_intensity(True)
    ref.advance_by(40)
    assert np.array_equal(bits(sim.read_electric()), bits(ref.read_electric()))
    assert np.array_equal(bits(sim.read_magnetic()), bits(ref.read_magnetic()))
    assert np.array_equal(bits(sim.read_intensity()), bits(ref.read_intensity()))
    naive = Simulation(scene, kernel=DP_KERNEL_NAIVE)
    assert naive.autotune()["candidates"] == 0


@pytest.mark.parametrize("extent", [(3, 5, 7), (5, 3, 3), (81, 7, 5), (130, 3, 2), (6, 9, 3)])
@pytest.mark.parametrize("kernel", [DP_KERNEL_FUSED, DP_KERNEL_NAIVE])
def test_written_fields_read_back_and_step_like_the_oracle(extent, kernel, threads):
    """Field writes and reads pass through the row packing whenever the
    device rows are padded (nx not a multiple of 4); these extents leave
    1, 2 or 3 rows after the last group of four.  Random fields written to
    both, read back unchanged, then stepped: the same bits."""
    scene = small_scene(extent)
    sim = Simulation(scene, kernel=kernel)
    ref = oracle.OracleSimulation(scene, threads=threads)
    rng = np.random.default_rng(sum(extent))
    count = 3 * int(np.prod(extent))
    e = rng.standard_normal(count).astype(np.float32)
    h = rng.standard_normal(count).astype(np.float32)
    sim.write_electric(e)
    sim.write_magnetic(h)
    assert np.array_equal(bits(sim.read_electric()), bits(e))
    assert np.array_equal(bits(sim.read_magnetic()), bits(h))
    ref.write_electric(e)
    ref.write_magnetic(h)
    sim.advance_by(7)
    ref.advance_by(7)
    assert np.array_equal(bits(sim.read_electric()), bits(ref.read_electric())), extent
    assert np.array_equal(bits(sim.read_magnetic()), bits(ref.read_magnetic())), extent


def test_a_tuned_plan_is_kept_for_its_grid_shape(threads):
    """dp_sim_autotune remembers the plan it picked for the grid's extent: a
    simulation created afterwards for a grid of that shape, with default
    options, starts from it, and exported and re-imported text gives the
    same plan; results stay bit-identical to the oracle either way."""
    from tests import scenes
    from diaphane_gb300.simulation import tuning_cache_clear, tuning_cache_export, tuning_cache_import
    tuning_cache_clear()
    scene, _ = scenes.graded()
    sim = Simulation(scene, kernel=DP_KERNEL_FUSED)
    sim.advance_by(5)
    tuned = sim.autotune(steps=2)
    plan = {k: tuned[k] for k in ("cells_per_lane", "tile_y", "ring_slots", "z_chunk")}
    assert sim.plan() == plan
    text = tuning_cache_export()
    assert len(text.splitlines()) == 1
    later = Simulation(scene, kernel=DP_KERNEL_FUSED)
    assert later.plan() == plan
    tuning_cache_clear()
    assert tuning_cache_export() == ""
    tuning_cache_import(text)
    again = Simulation(scene, kernel=DP_KERNEL_FUSED)
    assert again.plan() == plan
    again.advance_by(20)
    ref = oracle.OracleSimulation(scene, threads=threads)
    ref.advance_by(20)
    assert np.array_equal(bits(again.read_electric()), bits(ref.read_electric()))
    assert np.array_equal(bits(again.read_magnetic()), bits(ref.read_magnetic()))
    tuning_cache_clear()
