"""The FP64 instance: the same step in double on the GPU.  Against the
oracle's FP64 instance it must be bit-identical (same double expressions in
the same order, no contraction, IEEE division); the f32 step's error is then
measured against it."""
import numpy as np
import pytest

import oracle
from diaphane_gb300 import DP_KERNEL_FUSED, Simulation, Simulation64
from tests import scenes

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", sorted(scenes.PARITY_CASES))
def test_fp64_instance_matches_the_oracle_fp64(case, threads):
    scene, steps = scenes.PARITY_CASES[case]()
    reference = oracle.OracleSimulation(scene, fp64=True, threads=threads)
    gpu = Simulation64(scene)
    reference.advance_by(steps)
    gpu.advance_by(steps)
    assert gpu.step_count() == steps
    for name, ref, got in (("E", reference.read_electric(fp64=True), gpu.read_electric()),
                           ("H", reference.read_magnetic(fp64=True), gpu.read_magnetic())):
        assert np.abs(ref).max() > 0.0, name
        assert np.array_equal(ref.view(np.uint64), got.view(np.uint64)), f"{name} is not bit-identical"
    e_ref, e_gpu = reference.energy(), gpu.energy()
    assert e_gpu.total() == pytest.approx(e_ref.total(), rel=1e-12)


def test_f32_step_stays_close_to_fp64_while_the_pulse_flies():
    """Free flight 80³: the f32 fused step against the FP64 instance at step
    150, while the packet is inside the grid (by step 1000 it has left
    through the absorber and only a residue ~1e-5 of the peak remains, which
    makes "of peak" meaningless), as a fraction of the FP64 peak."""
    scene = scenes.free_flight(80)
    f32 = Simulation(scene, kernel=DP_KERNEL_FUSED)
    f64 = Simulation64(scene)
    f32.advance_by(150)
    f64.advance_by(150)
    for a, b in ((f32.read_electric(), f64.read_electric()), (f32.read_magnetic(), f64.read_magnetic())):
        peak = np.abs(b).max()
        assert peak > 0.0
        assert np.abs(a.astype(np.float64) - b).max() < 1e-3 * peak
