"""The total-field box (an extension of the reference's plane wave) on the
CUDA path: bit-identical to the oracle (the shared parity scenes include one),
one-way on every side, consistent across a restore (its incident line is
replayed to the restored step), and refused where it cannot run."""
import math

import numpy as np
import pytest

import oracle
from diaphane_gb300 import DP_KERNEL_FUSED, DP_KERNEL_NAIVE, Axis, Simulation, _abi
from tests import scenes
from tests.test_oracle_validation import box_scene

pytestmark = pytest.mark.gpu


def bits(a):
    return a.view(np.uint32)


@pytest.mark.parametrize("kernel", [DP_KERNEL_FUSED, DP_KERNEL_NAIVE])
def test_the_box_keeps_its_wave_inside_on_the_gpu(kernel):
    n, lo, hi = 48, 14, 34
    sim = Simulation(box_scene(Axis.Y, Axis.X, n, lo, hi), kernel=kernel)
    assert sim.kernel == kernel
    inside = np.zeros((n, n, n), dtype=bool)
    inside[lo:hi + 1, lo:hi + 1, lo:hi + 1] = True
    total_peak = scattered_peak = 0.0
    for _ in range(80):
        sim.advance_by(4)
        e = sim.read_electric().reshape(3, n, n, n)
        total_peak = max(total_peak, float(np.abs(e[0][inside]).max()))
        scattered_peak = max(scattered_peak, float(np.abs(e[:, ~inside]).max()))
    assert 0.8 <= total_peak < 1.25, total_peak
    assert 20.0 * math.log10(max(scattered_peak, 1e-30) / total_peak) < -80.0


def test_a_restore_replays_the_incident_line(threads):
    scene, _ = scenes.box_wave()
    straight = Simulation(scene)
    straight.advance_by(150)
    sim = Simulation(scene)
    sim.advance_by(60)
    snap = sim.snapshot()
    sim.advance_by(120)  # past the restore point and beyond, then back
    sim.restore(snap)
    sim.advance_by(90)
    assert sim.step_count() == 150
    assert np.array_equal(bits(sim.read_electric()), bits(straight.read_electric()))
    assert np.array_equal(bits(sim.read_magnetic()), bits(straight.read_magnetic()))
    ref = oracle.OracleSimulation(scene, threads=threads)
    ref.advance_by(150)
    assert np.array_equal(bits(sim.read_electric()), bits(ref.read_electric()))


def test_a_reset_starts_the_incident_line_over():
    scene, _ = scenes.box_wave()
    a = Simulation(scene)
    a.advance_by(70)
    first = a.read_electric()
    a.reset()
    a.advance_by(70)
    assert np.array_equal(bits(a.read_electric()), bits(first))


def test_the_box_does_not_run_backwards():
    scene, _ = scenes.box_wave()
    sim = Simulation(scene)
    sim.advance_by(5)
    with pytest.raises(_abi.DiaphaneError) as failure:
        sim.reverse_by(1)
    assert failure.value.status == _abi.DP_ERR_UNSUPPORTED



def test_a_restore_replays_from_a_line_checkpoint():
    # 700 steps leave checkpoints at 256 and 512; restoring to step 300
    # replays the line from 256, not from the start.
    scene, _ = scenes.box_wave()
    straight = Simulation(scene)
    straight.advance_by(700)
    sim = Simulation(scene)
    sim.advance_by(300)
    snap = sim.snapshot()
    sim.advance_by(400)
    sim.restore(snap)
    sim.advance_by(400)
    assert np.array_equal(bits(sim.read_electric()), bits(straight.read_electric()))
    assert np.array_equal(bits(sim.read_magnetic()), bits(straight.read_magnetic()))
