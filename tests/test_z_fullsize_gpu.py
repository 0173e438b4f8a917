"""Parity at the benchmark configurations' full size.

The reference's parity contract (tests/parity.rs:51-86) compares the two
solvers after a run; here it is applied, at 1000 steps, to the two plain
configurations the benchmark measures, at their full size, against the
oracle on every host core:

* the heterogeneous 512³ scene (200 dielectric spheres, a conducting sphere,
  a matched lossy slab, a total-field box, intensity on), and
* the 640×256×256 graded Bragg stack (x graded at cap 1.15 from 1 mm to
  0.1 mm, sheet source);

and, for the batched and served configurations, a sample of their own
scenes at their own sizes and step counts, through the batch and the served
loop, bit for bit against the oracle's solo runs.

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


def test_the_batched_configurations_scenes_at_their_own_size(threads):
    """The batched benchmark's scenes (seeds 0xBA7C0000 + k, axes
    log-uniform in [32, 160], 1000 steps): the first eight, advanced together
    in one batch with the benchmark's 50-step chunks, each bit-identical to
    the oracle's run of it alone."""
    from diaphane_gb300 import Batch
    scenes = [workloads.mixed_scene(0xBA7C_0000 + k) for k in range(8)]
    resolved = [ResolvedScene(s) for s in scenes]
    arena = int(1.05 * sum(Batch.bytes_for(r, STEPS) for r in resolved)) + (64 << 20)
    batch = Batch(arena, chunk_steps=50, max_scenes=8)
    ids = [batch.add(r, STEPS) for r in resolved]
    batch.run_to_completion()
    for k, (ident, scene) in enumerate(zip(ids, scenes)):
        reference = oracle.OracleSimulation(scene, threads=threads)
        reference.advance_by(STEPS)
        assert_identical(f"E of scene {k}", reference.read_electric(), batch.read_electric(ident))
        assert_identical(f"H of scene {k}", reference.read_magnetic(), batch.read_magnetic(ident))
    batch.close()


def test_the_served_configurations_requests_at_their_own_size(threads):
    """Requests of the served benchmark's default trace (48 at 16/s, axes in
    [48, 320], 200-5000 steps), at their own sizes and step counts: the five
    smallest by cell-updates are served together by continuous batching, and
    each one's probe series is the oracle's run of it alone, bit for bit."""
    from diaphane_gb300.serve import Server, poisson_trace
    trace = poisson_trace(48, 16.0)
    for r in trace:
        r.resolve()
    chosen = sorted(trace, key=lambda r: r.cells * r.steps)[:5]
    for r in chosen:
        r.arrival = 0.0
    server = Server(8 << 30, max_scenes=8, chunk_steps=50)
    server.serve(chosen)
    assert server.peak_active >= 2
    for r in chosen:
        assert r.outcome == "done"
        scene = workloads.mixed_scene(r.seed, r.lo, r.hi)
        reference = oracle.OracleSimulation(scene, threads=threads)
        expected = np.empty((r.steps, len(r.probes), 2), dtype=np.float32)
        for t in range(r.steps):
            reference.advance()
            for k, p in enumerate(r.probes):
                expected[t, k, 0] = reference.sample_electric(2, p)
                expected[t, k, 1] = reference.sample_magnetic(1, p)
        assert np.array_equal(r.series.view(np.uint32), expected.view(np.uint32)), r.ident
    server.close()
