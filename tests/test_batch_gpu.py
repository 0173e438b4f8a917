"""The batched form: every scene of a mixed batch must come out bit-identical
to its own solo run (and so to the oracle), whatever else shares the launch,
however the work is chunked, and whenever it joined."""
import numpy as np
import pytest

import oracle
from diaphane_gb300 import Batch, DP_KERNEL_NAIVE, ResolvedScene, Simulation, workloads
from tests import scenes

pytestmark = pytest.mark.gpu

ARENA = 4 << 30


def bits(a):
    return a.view(np.uint32)


def mixed(count, steps, seed0=1000, hi=72):
    return [ResolvedScene(workloads.mixed_scene(seed0 + k, lo=24, hi=hi)) for k in range(count)]


@pytest.mark.parametrize("graphs", [True, False])
def test_a_mixed_batch_matches_each_scene_run_alone(graphs):
    resolved = mixed(12, 120)
    batch = Batch(ARENA, chunk_steps=16, max_scenes=16, use_graphs=graphs)
    ids = [batch.add(r, 120 - 7 * k, accumulate_intensity=(k % 2 == 0)) for k, r in enumerate(resolved)]
    # Stored in the axis orders whose tiles cover the fewest cells: some of
    # these scenes are permuted, and must come out the same.
    assert any(batch.layout(ident)[0] != 0 for ident in ids)
    batch.run_to_completion()
    for k, (ident, r) in enumerate(zip(ids, resolved)):
        solo = Simulation(r, kernel=DP_KERNEL_NAIVE)
        solo.set_accumulate_intensity(k % 2 == 0)
        solo.advance_by(120 - 7 * k)
        assert batch.status(ident) == (120 - 7 * k, 120 - 7 * k)
        assert np.array_equal(bits(batch.read_electric(ident)), bits(solo.read_electric())), k
        assert np.array_equal(bits(batch.read_magnetic(ident)), bits(solo.read_magnetic())), k
        if k % 2 == 0:
            assert np.array_equal(bits(batch.read_intensity(ident)), bits(solo.read_intensity())), k


def test_scenes_that_join_and_leave_between_chunks(threads):
    """Continuous batching: a newcomer joins a running batch; results are the
    same as alone (checked against the oracle here)."""
    first, second = mixed(2, 0, seed0=2000)
    batch = Batch(ARENA, chunk_steps=10, max_scenes=4)
    a = batch.add(first, 95)
    for _ in range(4):
        batch.advance_chunk()
    b = batch.add(second, 60)       # joins at step 40 of the first
    batch.run_to_completion()
    for ident, r, steps in ((a, first, 95), (b, second, 60)):
        ref = oracle.OracleSimulation(r.scene, threads=threads)
        ref.advance_by(steps)
        assert np.array_equal(bits(batch.read_electric(ident)), bits(ref.read_electric()))
        assert np.array_equal(bits(batch.read_magnetic(ident)), bits(ref.read_magnetic()))
    batch.remove(a)
    used, cap = batch.memory()
    assert 0 < used < cap


def test_the_parity_scenes_in_one_batch(threads):
    cases = {name: make() for name, make in scenes.PARITY_CASES.items()}
    batch = Batch(ARENA, chunk_steps=50, max_scenes=16)
    ids = {name: batch.add(ResolvedScene(scene), steps) for name, (scene, steps) in cases.items()}
    batch.run_to_completion()
    for name, (scene, steps) in cases.items():
        ref = oracle.OracleSimulation(scene, threads=threads)
        ref.advance_by(steps)
        assert np.array_equal(bits(batch.read_electric(ids[name])), bits(ref.read_electric())), name
        assert np.array_equal(bits(batch.read_magnetic(ids[name])), bits(ref.read_magnetic())), name


def test_probes_record_ez_and_hy_every_step():
    (r,) = mixed(1, 0, seed0=3000)
    probes = [(5, 6, 7), (r.extent[0] // 2, r.extent[1] // 2, r.extent[2] // 2)]
    batch = Batch(ARENA, chunk_steps=8, max_scenes=2)
    ident = batch.add(r, 30, probes=probes)
    batch.run_to_completion()
    series = batch.read_probes(ident)
    assert series.shape == (30, 2, 2)
    solo = Simulation(r, kernel=DP_KERNEL_NAIVE)
    cells = r.cells
    for step in range(1, 31):
        solo.advance_by(1)
        e, h = solo.read_electric(), solo.read_magnetic()
        for k, (x, y, z) in enumerate(probes):
            i = (z * r.extent[1] + y) * r.extent[0] + x
            assert series[step - 1, k, 0] == e[2 * cells + i]
            assert series[step - 1, k, 1] == h[cells + i]


def test_admission_refuses_what_the_arena_cannot_hold():
    (r,) = mixed(1, 0, seed0=4000, hi=48)
    need = Batch.bytes_for(r, 100)
    batch = Batch(int(need * 2.5), chunk_steps=10, max_scenes=8)
    batch.add(r, 100)
    batch.add(r, 100)
    from diaphane_gb300 import DiaphaneError
    with pytest.raises(DiaphaneError) as err:
        batch.add(r, 100)
    assert err.value.name == "DP_ERR_OOM"
    # A probe series whose size would wrap is refused as unfittable, not
    # admitted at a wrapped small size; the batch carries on.
    big = Batch(int(need * 2.5), chunk_steps=10, max_scenes=8)
    with pytest.raises(DiaphaneError) as err:
        big.add(r, 1 << 62, probes=[(1, 1, 1)])
    assert err.value.name == "DP_ERR_OOM"
    ident = big.add(r, 20)
    big.run_to_completion()
    solo = Simulation(r)
    solo.advance_by(20)
    assert np.array_equal(bits(big.read_electric(ident)), bits(solo.read_electric()))


def test_a_refused_admission_leaves_the_arena_as_it_was():
    from diaphane_gb300 import DiaphaneError
    (r,) = mixed(1, 0, seed0=4100, hi=48)
    batch = Batch(ARENA, chunk_steps=10, max_scenes=4)
    ident = batch.add(r, 20)
    used = batch.memory()[0]
    with pytest.raises(DiaphaneError) as err:
        batch.add(r, 20, probes=[(1, 1, 1), (r.extent[0], 0, 0)])  # the second probe lies outside
    assert err.value.name == "DP_ERR_RANGE"
    assert batch.memory()[0] == used
    batch.run_to_completion()
    solo = Simulation(r)
    solo.advance_by(20)
    assert np.array_equal(bits(batch.read_electric(ident)), bits(solo.read_electric()))


def test_reads_into_a_caller_buffer_match_fresh_arrays():
    import torch
    resolved = mixed(3, 30)
    batch = Batch(ARENA, chunk_steps=16, max_scenes=4)
    ids = [batch.add(r, 30, accumulate_intensity=True) for r in resolved]
    batch.run_to_completion()
    pinned = torch.empty(3 * max(r.cells for r in resolved) + 5, dtype=torch.float32, pin_memory=True).numpy()
    for ident, r in zip(ids, resolved):
        solo = Simulation(r)
        solo.set_accumulate_intensity(True)
        solo.advance_by(30)
        for read_batch, read_solo in [(batch.read_electric, solo.read_electric),
                                      (batch.read_magnetic, solo.read_magnetic),
                                      (batch.read_intensity, solo.read_intensity)]:
            fresh = read_batch(ident)
            into = read_batch(ident, out=pinned)
            assert into.size == fresh.size and np.shares_memory(into, pinned)
            assert np.array_equal(bits(into), bits(fresh))
            assert np.array_equal(bits(read_solo(out=pinned)), bits(fresh))


def test_a_total_field_box_in_a_batch_matches_its_solo_run(threads):
    # The box's side faces read per-step profiles the batch stages per chunk;
    # mixed with other scenes and split over several chunks, it must still
    # come out bit-identical to its solo run and to the oracle.
    scene, steps = scenes.box_wave()
    others = mixed(3, steps, seed0=4000)
    batch = Batch(ARENA, chunk_steps=32, max_scenes=8)
    box = batch.add(ResolvedScene(scene), steps, accumulate_intensity=True)
    ids = [batch.add(r, steps - 11 * k) for k, r in enumerate(others)]
    batch.run_to_completion()
    solo = Simulation(scene)
    solo.set_accumulate_intensity(True)
    solo.advance_by(steps)
    assert np.array_equal(bits(batch.read_electric(box)), bits(solo.read_electric()))
    assert np.array_equal(bits(batch.read_magnetic(box)), bits(solo.read_magnetic()))
    assert np.array_equal(bits(batch.read_intensity(box)), bits(solo.read_intensity()))
    ref = oracle.OracleSimulation(scene, threads=threads)
    ref.advance_by(steps)
    assert np.array_equal(bits(batch.read_electric(box)), bits(ref.read_electric()))
    for k, (ident, r) in enumerate(zip(ids, others)):
        alone = Simulation(r)
        alone.advance_by(steps - 11 * k)
        assert np.array_equal(bits(batch.read_electric(ident)), bits(alone.read_electric())), k


def order_scenes():
    """Scenes with three different extents, so every axis order moves them:
    lossy absorbers and materials, a graded grid (gains that differ per
    axis), point sources of two polarizations (one moving) and a plane wave."""
    from diaphane_gb300 import Axis, Boundary, Extent, Scene, Source, Waveform
    several = Scene.empty(Extent(40, 28, 34), 1e-3).with_boundary(Boundary.absorbing(8, 1e-6))
    frequency = several.grid.frequency_for_resolution(20.0)
    several.sources.append(Source.point((0.0, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    several.sources.append(Source.point((1e-3, -2e-3, 0.0), Axis.X, Waveform.ricker(frequency)).with_amplitude(-0.5))
    several.sources.append(Source.point_moving((-6e-3, 2e-3, 0.0), (2.7e8, 0.0, 0.0), Axis.Y,
                                               Waveform.ricker(frequency)))
    made = [several, scenes.materials()[0], scenes.graded()[0], scenes.plane_wave()[0]]
    return [ResolvedScene(s) for s in made] + mixed(2, 0, seed0=5000, hi=60)


@pytest.mark.parametrize("order", range(1, 7))
def test_every_axis_order_gives_each_scene_its_own_results(order):
    """A batch may store a scene with its axes permuted, for fewer idle lanes;
    forced into each of the six orders, every scene's fields, intensity and
    probe series still equal its solo run's bit for bit."""
    from diaphane_gb300 import Axis
    resolved = order_scenes()
    steps = 45

    def probes(r):
        return [(3, 4, 5), (r.extent[0] - 2, r.extent[1] // 2, r.extent[2] - 3)]

    batch = Batch(ARENA, chunk_steps=16, max_scenes=8, axis_order=order)
    ids = [batch.add(r, steps, accumulate_intensity=True, probes=probes(r)) for r in resolved]
    for ident in ids:
        stored, width = batch.layout(ident)
        assert stored == order - 1 and width in (32, 64, 128)
        assert stored in (0, 2) or width == 32  # the scene's x elsewhere than x: 32-wide tiles
    batch.run_to_completion()
    for k, (ident, r) in enumerate(zip(ids, resolved)):
        solo = Simulation(r, kernel=DP_KERNEL_NAIVE)
        solo.set_accumulate_intensity(True)
        expected = np.zeros((steps, 2, 2), np.float32)
        for step in range(steps):
            solo.advance_by(1)
            for j, p in enumerate(probes(r)):
                expected[step, j] = solo.sample_electric(Axis.Z, p), solo.sample_magnetic(Axis.Y, p)
        assert np.array_equal(bits(batch.read_probes(ident)), bits(expected)), k
        assert np.array_equal(bits(batch.read_electric(ident)), bits(solo.read_electric())), k
        assert np.array_equal(bits(batch.read_magnetic(ident)), bits(solo.read_magnetic())), k
        assert np.array_equal(bits(batch.read_intensity(ident)), bits(solo.read_intensity())), k
