"""The benchmark workloads on the host: the heterogeneous scene resolves at
every size the benchmark and the tests use (the total-field box must fit
inside the grid and outside the absorber), its box faces sit where the
benchmark line says (cells 26 and 485 at 512), and the seeded scenes are the
same scene for the same seed."""
import math

import numpy as np
import pytest

from diaphane_gb300 import ResolvedScene, workloads
from diaphane_gb300._abi import DP_TABLE_COEFFICIENTS


def box_cells(scene):
    (source,) = scene.sources
    lo = scene.grid.to_cell(source.box_low)
    hi = scene.grid.to_cell(source.box_high)
    return [math.floor(v) for v in lo], [math.floor(v) for v in hi]


@pytest.mark.parametrize("side", [24, 32, 48, 64, 96, 256, 512])
def test_the_heterogeneous_scene_resolves_with_its_box_inside_the_grid(side):
    scene = workloads.heterogeneous(side)
    resolved = ResolvedScene(scene)
    assert tuple(resolved.extent) == (side, side, side)
    lo, hi = box_cells(scene)
    for a in range(3):
        assert 1 <= lo[a] < hi[a] <= side - 2
        if side >= 64:
            assert lo[a] >= 10 and hi[a] <= side - 11  # outside the 10-cell absorber


def test_the_benchmark_box_faces_are_at_cells_26_and_485():
    lo, hi = box_cells(workloads.heterogeneous(512))
    assert lo == [26, 26, 26] and hi == [485, 485, 485]


def test_seeded_scenes_repeat():
    a = ResolvedScene(workloads.heterogeneous(48, seed=7)).table(DP_TABLE_COEFFICIENTS)
    b = ResolvedScene(workloads.heterogeneous(48, seed=7)).table(DP_TABLE_COEFFICIENTS)
    c = ResolvedScene(workloads.heterogeneous(48, seed=8)).table(DP_TABLE_COEFFICIENTS)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))
    assert not np.array_equal(a, c)


@pytest.mark.parametrize("seed", [0xBA7C_0000 + k for k in range(6)])
def test_mixed_batch_scenes_resolve_with_axes_in_range(seed):
    resolved = ResolvedScene(workloads.mixed_scene(seed))
    assert all(32 <= n <= 160 for n in resolved.extent)
    again = ResolvedScene(workloads.mixed_scene(seed))
    assert tuple(again.extent) == tuple(resolved.extent)
