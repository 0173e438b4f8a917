"""The simulation API's behaviour on the device: reset, refusal to reverse a
lossy scene, snapshot/restore, the timeline scrub, zero-copy pointers."""
import numpy as np
import pytest

from diaphane_gb300 import (Boundary, DiaphaneError, Extent, Scene, Simulation, Timeline, _abi)
from tests import scenes

pytestmark = pytest.mark.gpu


def test_resetting_clears_the_device_buffers():
    """tests/parity.rs:385-404."""
    sim = Simulation(Scene.photon(Extent.cube(32)))
    sim.advance_by(120)
    assert np.any(sim.read_electric() != 0)
    sim.reset()
    assert sim.step_count() == 0
    assert np.all(sim.read_electric() == 0) and np.all(sim.read_magnetic() == 0)


def test_reversal_refuses_a_lossy_scene():
    """src/cpu.rs:970-997: an absorber makes the scene irreversible."""
    sim = Simulation(Scene.photon(Extent.cube(32)))
    assert not sim.is_reversible()
    sim.advance()
    with pytest.raises(DiaphaneError) as err:
        sim.reverse()
    assert err.value.name == "DP_ERR_LOSSY"


def test_reversal_refuses_to_pass_the_start():
    sim = Simulation(scenes.reversible())
    sim.advance_by(3)
    with pytest.raises(DiaphaneError) as err:
        sim.reverse_by(4)
    assert err.value.name == "DP_ERR_RANGE"


def test_reversing_all_the_way_returns_to_an_empty_domain():
    """src/cpu.rs:952-968 on the device."""
    scene = Scene.photon(Extent.cube(24)).with_boundary(Boundary.PEC)
    sim = Simulation(scene)
    sim.advance_by(120)
    excited = sim.energy().total()
    sim.reverse_by(120)
    assert sim.step_count() == 0
    assert sim.energy().total() < excited * 1e-8


def test_a_timeline_scrubs_the_gpu_solver():
    """tests/parity.rs:406-445."""
    scene = Scene.photon(Extent.cube(32))
    reference = Simulation(scene)
    reference.advance_by(70)
    expected = reference.read_electric()
    sim = Simulation(scene)
    timeline = Timeline(25, 8)
    for _ in range(120):
        sim.advance_by(1)
        timeline.observe(sim)
    assert timeline.keyframe_count() > 1
    outcome = timeline.seek(sim, 70)
    assert sim.step_count() == 70 and outcome.kind == "keyframe"
    scrubbed = sim.read_electric()
    assert np.array_equal(expected.view(np.uint32), scrubbed.view(np.uint32))


def test_snapshot_restore_round_trip_and_size_checks():
    sim = Simulation(Scene.photon(Extent.cube(24)))
    sim.advance_by(40)
    snap = sim.snapshot()
    assert snap.bytes() == 24 * 24 ** 3
    sim.advance_by(10)
    sim.restore(snap)
    assert sim.step_count() == 40
    assert np.array_equal(sim.read_electric(), snap.electric)
    with pytest.raises(DiaphaneError):
        sim.write_electric(np.zeros(10, np.float32))


def test_device_pointer_and_bytes_per_step():
    sim = Simulation(Scene.photon(Extent.cube(24)))
    assert sim.bytes_per_step() == 48 * 24 ** 3
    assert sim.field_bytes() == 12 * 24 ** 3
    assert sim.device_ptr(_abi.DP_FIELD_ELECTRIC) != 0
    sim.advance_by(5)
    sim.wait(10_000)
    assert sim.launch_count() > 0


def test_grids_whose_rows_are_not_a_multiple_of_4_cells_run_fused_with_a_pitch():
    """nx = 81: the device rows are padded to 84 cells; reads, writes and
    restores go through the dense host layout unchanged."""
    from tests import scenes
    import oracle
    scene, steps = scenes.graded()
    sim = Simulation(scene)
    assert sim.kernel == 1 and sim.extent[0] == 81
    assert _abi.lib().dp_sim_row_pitch(sim.handle) == 84
    sim.advance_by(40)
    snap = sim.snapshot()
    sim.advance_by(10)
    sim.restore(snap)
    sim.advance_by(10)
    ref = oracle.OracleSimulation(scene, threads=8)
    ref.advance_by(50)
    assert np.array_equal(sim.read_electric().view(np.uint32), ref.read_electric().view(np.uint32))
