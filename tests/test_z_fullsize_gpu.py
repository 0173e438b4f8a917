"""Parity at the benchmark configurations' full size.

The reference's parity contract (tests/parity.rs:51-86) compares the two
solvers after a run; here it is applied, at 1000 steps, to the two plain
configurations the benchmark measures, at their full size, against the
oracle on every host core:

* the heterogeneous 512³ scene (200 dielectric spheres, a conducting sphere,
  a matched lossy slab, a total-field box, intensity on), and
* the 640×256×256 graded Bragg stack (x graded at cap 1.15 from 1 mm to
  0.1 mm, sheet source).

Tolerance: at most 1e-5 of the all-component peak for E and H, and the
stronger expectation the smaller parity scenes already meet: E, H and the
intensity bit-identical, since both sides evaluate the same f32 expressions
in the same order with no contraction and IEEE division.

These run for about three minutes (the oracle needs roughly 110 ms per 512³
step on 16 cores), so they sit near the end of the collection order.
"""
import numpy as np
import pytest

import oracle
from diaphane_gb300 import DP_KERNEL_FUSED, ResolvedScene, Simulation, workloads
from tests.helpers import assert_field_parity

pytestmark = pytest.mark.gpu

STEPS = 1000
TOLERANCE = 1e-5


def run_both(scene, steps: int, intensity: bool, threads: int):
    resolved = ResolvedScene(scene)
    candidate = Simulation(resolved)
    assert candidate.kernel == DP_KERNEL_FUSED
    candidate.set_accumulate_intensity(intensity)
    candidate.advance_by(steps)  # queued on the GPU; the oracle runs meanwhile
    reference = oracle.OracleSimulation(scene, threads=threads)
    reference.set_accumulate_intensity(intensity)
    reference.advance_by(steps)
    candidate.wait(600_000)
    assert reference.step_count() == candidate.step_count() == steps
    return reference, candidate


def assert_identical(name: str, a: np.ndarray, b: np.ndarray) -> None:
    same = a.view(np.uint32) == b.view(np.uint32)
    if not same.all():
        bad = int(np.count_nonzero(~same))
        first = int(np.argmin(same))
        pytest.fail(f"{name}: {bad} of {a.size} values differ, first at {first}: {a[first]!r} vs {b[first]!r}")


def check(reference, candidate, steps: int, intensity: bool) -> None:
    cells = candidate.cells
    assert candidate.is_finite() and reference.is_finite()
    e_ref, e_gpu = reference.read_electric(), candidate.read_electric()
    assert_field_parity("E", e_ref, e_gpu, cells, steps, TOLERANCE)
    assert_identical("E", e_ref, e_gpu)
    del e_ref, e_gpu
    h_ref, h_gpu = reference.read_magnetic(), candidate.read_magnetic()
    assert_field_parity("H", h_ref, h_gpu, cells, steps, TOLERANCE)
    assert_identical("H", h_ref, h_gpu)
    del h_ref, h_gpu
    if intensity:
        i_ref, i_gpu = reference.read_intensity(), candidate.read_intensity()
        assert i_ref.max() > 0
        assert_identical("intensity", i_ref, i_gpu)


def test_heterogeneous_512_after_1000_steps(threads):
    """The benchmark's own scene and grid, intensity on."""
    scene = workloads.heterogeneous(512)
    reference, candidate = run_both(scene, STEPS, True, threads)
    assert candidate.extent == (512, 512, 512)
    check(reference, candidate, STEPS, True)


def test_graded_stack_640x256x256_after_1000_steps(threads):
    """The graded Bragg stack at full size: the fused path's per-cell x gains
    on a grid graded down to a tenth of its coarse cell."""
    scene = workloads.graded_stack()
    reference, candidate = run_both(scene, STEPS, False, threads)
    assert candidate.extent == (640, 256, 256)
    check(reference, candidate, STEPS, False)
