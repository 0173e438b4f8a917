"""The product's host setup (dp_scene_*) against the oracle's restatement of
the reference setup: every table a kernel reads, and every step's injections,
must agree bit for bit."""
import numpy as np
import pytest

import oracle
from diaphane_gb300 import _abi, Axis, Extent, ResolvedScene, Scene
from tests import scenes

TABLES = [_abi.DP_TABLE_MAGNETIC_GAINS, _abi.DP_TABLE_ELECTRIC_GAINS, _abi.DP_TABLE_CELL_CENTERS,
          _abi.DP_TABLE_ABSORBER, _abi.DP_TABLE_COEFFICIENTS, _abi.DP_TABLE_MATERIAL_INDEX,
          _abi.DP_TABLE_PRIMARY, _abi.DP_TABLE_DUAL]


def all_scenes():
    out = {name: make()[0] for name, make in scenes.PARITY_CASES.items()}
    out["reversible"] = scenes.reversible()
    out["free_flight"] = scenes.free_flight(40)
    return out


@pytest.mark.parametrize("name", sorted(all_scenes()))
def test_tables_match_the_oracle_bit_for_bit(name):
    scene = all_scenes()[name]
    product = ResolvedScene(scene)
    reference = oracle.OracleSimulation(scene)
    assert product.extent == reference.extent
    assert np.float32(product.time_step) == np.float32(reference.time_step())
    for table in TABLES:
        a, b = product.table(table), reference.table(table)
        if table == _abi.DP_TABLE_MATERIAL_INDEX:
            a = a.astype(np.uint32)
        assert a.shape == b.shape, table
        assert np.array_equal(a.view(np.uint32) if a.dtype == np.float32 else a,
                              b.view(np.uint32) if b.dtype == np.float32 else b), f"table {table} differs"
    assert product.reversible == reference.is_reversible()
    assert np.float32(product.absorber_peak) == np.float32(reference.absorber_peak())


@pytest.mark.parametrize("name", sorted(n for n, s in all_scenes().items() if not scenes.has_box(s)))
def test_injections_match_the_oracle_at_every_step(name):
    scene = all_scenes()[name]
    product = ResolvedScene(scene)
    reference = oracle.OracleSimulation(scene)
    dt = np.float32(product.time_step)
    for step in list(range(0, 400, 7)) + [1000]:
        time = float(np.float32(step + 1) * dt)
        a, b = product.injections(time), reference.injections(time)
        assert len(a) == len(b)
        for x, y in zip(a, b):
            assert tuple(x.origin) == tuple(y.origin) and tuple(x.extent) == tuple(y.extent)
            assert x.component == y.component and x.magnetic == y.magnetic
            assert np.float32(x.value).view(np.uint32) == np.float32(y.value).view(np.uint32)
            assert np.float32(x.inverse_waist_squared) == np.float32(y.inverse_waist_squared)


def test_material_index_uses_last_shape_and_culls_nothing():
    """Overlapping shapes paint in order; the product rasterizes by bounding
    range, and that must change nothing against the all-cells scan."""
    from diaphane_gb300 import Material, Shape
    rng = np.random.default_rng(7)
    scene = Scene.empty(Extent(50, 44, 38), 1e-3)
    for i in range(40):
        m = scene.materials.push(Material.dielectric(1.0 + 0.05 * i))
        c = tuple(float(v) for v in rng.uniform(-0.02, 0.02, 3))
        kind = i % 3
        if kind == 0:
            scene.shapes.append(Shape.sphere(c, float(rng.uniform(1e-3, 9e-3)), m))
        elif kind == 1:
            scene.shapes.append(Shape.block(c, tuple(float(v) for v in rng.uniform(1e-3, 2e-2, 3)), m))
        else:
            scene.shapes.append(Shape.slab(Axis(i % 3), c[0], float(rng.uniform(1e-3, 6e-3)), m))
    a = ResolvedScene(scene).table(_abi.DP_TABLE_MATERIAL_INDEX).astype(np.uint32)
    b = oracle.OracleSimulation(scene).table(_abi.DP_TABLE_MATERIAL_INDEX)
    assert np.array_equal(a, b)
    assert len(np.unique(a)) > 10


def many_materials(count, side=20):
    """`count` materials, each painted on its own small cube somewhere in the grid."""
    from diaphane_gb300 import Boundary, Material, Shape
    scene = Scene.empty(Extent.cube(side), 1e-3).with_boundary(Boundary.PEC)
    for i in range(count - 1):
        m = scene.materials.push(Material.dielectric(1.5 + 0.001 * i))
        x, y, z = (i * 7) % side, (i * 11) % side, (i * 13) % side
        centre = [(c - side / 2 + 0.5) * 1e-3 for c in (x, y, z)]
        scene.shapes.append(Shape.block(centre, (1e-3, 1e-3, 1e-3), m))
    return scene


def test_past_256_materials_the_index_widens_to_u16():
    scene = many_materials(300)
    resolved = ResolvedScene(scene)
    assert resolved.index_bytes == 2 and resolved.material_count == 300
    ours = resolved.table(_abi.DP_TABLE_MATERIAL_INDEX)
    assert ours.dtype == np.uint16
    theirs = oracle.OracleSimulation(scene).table(_abi.DP_TABLE_MATERIAL_INDEX)
    assert np.array_equal(ours.astype(np.uint32), theirs)
    assert ours.max() > 255


def test_more_than_65536_materials_is_rejected():
    from diaphane_gb300 import Boundary, DiaphaneError, Material
    scene = Scene.empty(Extent.cube(4), 1e-3).with_boundary(Boundary.PEC)
    # 65537 distinct entries (pushing them one by one would merge-check each).
    scene.materials.materials += [Material.dielectric(1.0 + 1e-5 * (i + 1)) for i in range(65536)]
    with pytest.raises(DiaphaneError) as err:
        ResolvedScene(scene)
    assert err.value.name == "DP_ERR_UNSUPPORTED"


@pytest.mark.parametrize("case", ["graded", "photon"])
def test_world_to_cell_lookup_matches_the_oracles_coordinate_map(case):
    """Grid::cell_lookup (src/grid.rs:635-646) against the oracle's own
    world-to-cell map, sample for sample."""
    scene = scenes.graded()[0] if case == "graded" else scenes.photon()[0]
    resolved = ResolvedScene(scene)
    samples = resolved.lookup_samples()
    assert samples == min(max(4 * max(resolved.extent), 256), 8192)
    ours = resolved.cell_lookup()
    size = oracle.grid_resolve(scene.grid)["size"]
    expected = np.empty(3 * samples, np.float32)
    for k in range(samples):
        fraction = np.float32(k) / np.float32(samples - 1)
        position = [(fraction - np.float32(0.5)) * np.float32(size[a]) for a in range(3)]
        cell = oracle.grid_map(scene.grid, _abi.DP_MAP_TO_CELL, position)
        for a in range(3):
            expected[a * samples + k] = cell[a]
    assert np.array_equal(ours.view(np.uint32), expected.view(np.uint32))


def test_a_total_field_box_is_not_a_function_of_time_alone():
    # Its corrections come from the incident line's history, so the
    # stateless per-time query refuses it on both sides.
    scene, _ = scenes.box_wave()
    with pytest.raises(Exception):
        ResolvedScene(scene).injections(1e-12)
    with pytest.raises(Exception):
        oracle.OracleSimulation(scene).injections(1e-12)
