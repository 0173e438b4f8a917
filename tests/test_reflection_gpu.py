"""The reference's reflection figures measured through the CUDA path.

The absorbing layer's reflection (tests/validation.rs:484-550, about -58 dB)
and a grading transition's (tests/graded.rs:266-313, -32.5 dB at cap 1.15 and
-52.4 dB at 1.05) come from probe traces of a Ricker pulse; here the traces
are recorded by the fused step on the GPU, checked bit for bit against the
oracle's, and the figures computed from them: the dB the product delivers,
not only the oracle's."""
import math

import numpy as np
import pytest

import oracle
from diaphane_gb300 import Axis, Extent, Grid, Refinement, Scene, Simulation, Source, Waveform
from diaphane_gb300._abi import DP_KERNEL_FUSED

pytestmark = pytest.mark.gpu

CELL, FINE = 1e-3, 0.25e-3
DOMAIN = (0.096, 0.040, 0.040)


def traces(scene, probe, steps, threads):
    """Ez at `probe` after every step, on the fused GPU step and the oracle."""
    sim = Simulation(scene, kernel=DP_KERNEL_FUSED)
    ref = oracle.OracleSimulation(scene, threads=threads)
    gpu, cpu = [], []
    for _ in range(steps):
        sim.advance()
        ref.advance()
        gpu.append(sim.sample_electric(Axis.Z, probe))
        cpu.append(ref.sample_electric(Axis.Z, probe))
    sim.close()
    gpu, cpu = np.array(gpu, np.float32), np.array(cpu, np.float32)
    assert np.array_equal(gpu.view(np.uint32), cpu.view(np.uint32))
    return gpu


def absorber_trace(length, steps, threads):
    scene = Scene.empty(Extent(length, 40, 40), 1e-3)
    frequency = scene.grid.frequency_for_resolution(20.0)
    position = oracle.grid_map(scene.grid, 1, (20.5, 20.0, 20.0))
    scene.sources.append(Source.point(position, Axis.Z, Waveform.ricker(frequency)))
    return traces(scene, (36, 20, 20), steps, threads)


def test_the_absorbing_layer_reflects_58_db_down_on_the_gpu(threads):
    near, far = absorber_trace(72, 380, threads), absorber_trace(200, 380, threads)
    decibels = 20.0 * math.log10(float(np.abs(near - far).max()) / float(np.abs(far).max()))
    assert -61.0 < decibels < -55.0, decibels  # the reference reports about -58 dB


def graded_trace(grid, steps, threads):
    scene = Scene.on_grid(grid)
    frequency = scene.grid.frequency_for_resolution(20.0)
    scene.sources.append(Source.point((-0.012, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    probe = tuple(int(v) for v in oracle.grid_map(grid, 2, (-0.004, 0.0, 0.0)))
    return traces(scene, probe, steps, threads)


def test_a_grading_transition_reflects_as_published_on_the_gpu(threads):
    fine = graded_trace(Grid.graded(DOMAIN, 1.0 / CELL, [Refinement.across(Axis.X, 0.0, 2.0 * DOMAIN[0], FINE)]),
                        340, threads)
    incident = float(np.abs(fine).max())

    def decibels(cap):
        band = Refinement.across(Axis.X, 0.0, 0.028, FINE)
        graded = graded_trace(Grid.graded(DOMAIN, 1.0 / CELL, [band], cap), 340, threads)
        return 20.0 * math.log10(float(np.abs(graded - fine).max()) / incident)

    default, gentle = decibels(1.15), decibels(1.05)
    assert abs(default - (-32.5)) < 1.5 and abs(gentle - (-52.4)) < 1.5, (default, gentle)
    assert gentle < default - 3.0
