"""Keyframes in device memory, per-step probes and asynchronous read-back on
the single-scene handle.

The device timeline must make the reference Timeline's decisions
(src/timeline.rs:137-212, its tests at :215-330) and land on states
bit-identical to a fresh run; probes must equal the oracle's per-step
samples; an asynchronous read must equal the synchronous one."""
import numpy as np
import pytest
import torch

import oracle
from diaphane_gb300 import (DeviceTimeline, DiaphaneError, Extent, Scene, Simulation, Timeline, _abi, workloads)
from tests import scenes

pytestmark = pytest.mark.gpu


def bits(a):
    return a.view(np.uint32)


def fresh(scene, steps):
    sim = Simulation(scene)
    sim.advance_by(steps)
    return sim.read_electric(), sim.read_magnetic()


def test_device_timeline_makes_the_host_timelines_decisions():
    """The same observe/seek script on a host timeline and a device one:
    identical Seek outcomes, identical fields, and both equal to a fresh run
    to the target."""
    scene, _ = scenes.materials()
    host_sim, dev_sim = Simulation(scene), Simulation(scene)
    host, dev = Timeline(20, 3), DeviceTimeline(dev_sim, 20, 3)
    # Batches that do not divide the interval, as a viewer's would.
    for _ in range(17):
        for sim, tl in ((host_sim, host), (dev_sim, dev)):
            sim.advance_by(7)
            tl.observe(sim)
    assert dev.keyframe_count() == host.keyframe_count() == 3
    assert dev.earliest() == host.earliest()
    assert dev.bytes() == host.bytes() == 3 * 24 * dev_sim.cells
    for target in (100, 75, 119, 30, 5, 118, 118, 60):
        a, b = host.seek(host_sim, target), dev.seek(dev_sim, target)
        assert (a.kind, a.replayed, a.at) == (b.kind, b.replayed, b.at), target
        assert dev_sim.step_count() == target
        e, h = fresh(scene, target)
        assert np.array_equal(bits(dev_sim.read_electric()), bits(e)), target
        assert np.array_equal(bits(dev_sim.read_magnetic()), bits(h)), target
        assert np.array_equal(bits(host_sim.read_electric()), bits(e)), target
        host.observe(host_sim)
        dev.observe(dev_sim)


def test_the_window_slides_and_falls_back_to_the_start():
    """src/timeline.rs:258-289: an old target beyond the window replays from
    zero; clearing forgets every keyframe."""
    scene = Scene.photon(Extent.cube(24))
    sim = Simulation(scene)
    tl = DeviceTimeline(sim, 10, 2)
    for _ in range(60):
        sim.advance_by(1)
        tl.observe(sim)
    assert tl.keyframe_count() == 2 and tl.earliest() == 50
    outcome = tl.seek(sim, 15)
    assert outcome.kind == "start" and outcome.replayed == 15
    e, _ = fresh(scene, 15)
    assert np.array_equal(bits(sim.read_electric()), bits(e))
    assert tl.seek(sim, 15).kind == "unchanged"
    assert tl.seek(sim, 40).kind == "forward"
    outcome = tl.seek(sim, 55)
    assert outcome.kind == "forward"
    outcome = tl.seek(sim, 52)
    assert (outcome.kind, outcome.at, outcome.replayed) == ("keyframe", 50, 2)
    tl.clear()
    assert tl.keyframe_count() == 0 and tl.earliest() is None and tl.bytes() == 0
    assert tl.seek(sim, 3).kind == "start"


def test_seeking_restarts_the_intensity_average():
    scene = Scene.photon(Extent.cube(24))
    sim = Simulation(scene)
    sim.set_accumulate_intensity(True)
    tl = DeviceTimeline(sim, 10, 4)
    for _ in range(4):
        sim.advance_by(10)
        tl.observe(sim)
    tl.seek(sim, 25)
    assert sim.accumulated_steps() == 5  # replayed from the keyframe at 20
    with pytest.raises(ValueError):
        tl.observe(Simulation(scene))


def test_probes_record_every_step_like_the_oracle(threads):
    scene = workloads.mixed_scene(7, lo=36, hi=48)
    sim = Simulation(scene)
    n = sim.extent
    cells = [(n[0] // 2, n[1] // 2, n[2] // 2), (3, 4, 5), (n[0] - 1, n[1] - 1, n[2] - 1), (n[0] // 3, 1, n[2] // 4)]
    sim.set_probes(cells, capacity=64)
    ref = oracle.OracleSimulation(scene, threads=threads)
    expected = np.empty((150, len(cells), 2), np.float32)
    for t in range(150):
        ref.advance()
        for k, c in enumerate(cells):
            expected[t, k] = (ref.sample_electric(2, c), ref.sample_magnetic(1, c))
    sim.advance_by(150)
    got = sim.read_probes(87, 64)  # the whole ring: steps 87..150
    assert np.array_equal(bits(got), bits(expected[86:150]))
    assert np.array_equal(bits(sim.read_probes(140, 5)), bits(expected[139:144]))
    with pytest.raises(DiaphaneError):
        sim.read_probes(86, 1)   # overwritten
    with pytest.raises(DiaphaneError):
        sim.read_probes(150, 2)  # not yet taken
    sim.reset()
    with pytest.raises(DiaphaneError):
        sim.read_probes(140, 1)  # belongs to the abandoned history
    sim.advance_by(3)
    assert np.array_equal(bits(sim.read_probes(1, 3)), bits(expected[0:3]))
    with pytest.raises(DiaphaneError):
        sim.set_probes([(n[0], 0, 0)], 8)
    # A ring whose byte count would wrap is refused before anything changes:
    # the current probes keep recording.
    with pytest.raises(DiaphaneError) as err:
        sim.set_probes(cells, 1 << 62)
    assert err.value.status == _abi.DP_ERR_OOM
    sim.advance_by(2)
    assert np.array_equal(bits(sim.read_probes(4, 2)), bits(expected[3:5]))


def test_asynchronous_read_matches_the_synchronous_one():
    scene = workloads.mixed_scene(3, lo=40, hi=60)
    sim = Simulation(scene)
    sim.set_accumulate_intensity(True)
    sim.advance_by(80)
    pinned = torch.empty(3 * sim.cells, dtype=torch.float32, pin_memory=True)
    sim.read_field_async(_abi.DP_FIELD_ELECTRIC, pinned.data_ptr(), pinned.numel())
    sim.advance_by(5)  # queued behind the copy
    sim.wait()
    early = pinned.numpy().copy()
    check = Simulation(scene)
    check.advance_by(80)
    assert np.array_equal(bits(early), bits(check.read_electric()))
