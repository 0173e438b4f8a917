"""Scene rasterization on the GPU (Scene::material_indices, src/scene.rs:181-206)
against the oracle's restatement: the u8 index must be identical cell for
cell, padding bytes zero, whatever the row pitch."""
import numpy as np
import pytest
import torch

import oracle
from diaphane_gb300 import Axis, Extent, Material, ResolvedScene, Scene, Shape, _abi, workloads
from tests import scenes

pytestmark = pytest.mark.gpu


def device_index(resolved, pitch):
    nx, ny, nz = resolved.extent
    dtype = torch.uint8 if resolved.index_bytes == 1 else torch.int16
    buf = torch.full((nz * ny * pitch,), 0x2B, dtype=dtype, device="cuda")
    resolved.rasterize(buf.data_ptr(), pitch)
    torch.cuda.synchronize()
    out = buf.cpu().numpy()
    if resolved.index_bytes == 2:
        out = out.view(np.uint16)
    return out.reshape(nz * ny, pitch)


def blocks_and_slabs():
    scene = Scene.photon(Extent(45, 38, 29))
    a = scene.materials.push(Material.dielectric(2.0))
    b = scene.materials.push(Material.dielectric(3.0))
    c = scene.materials.push(Material.PERFECT_CONDUCTOR)
    scene.shapes += [Shape.block((0.004, -0.002, 0.0), (0.011, 0.017, 0.009), a),
                     Shape.slab(Axis.Y, 0.003, 0.006, b),
                     Shape.sphere((-0.006, 0.004, 0.002), 0.0071, c),
                     Shape.block((0.0, 0.0, 0.0), (1.0, 1.0, 0.0), a)]  # zero thickness: the centre plane at most
    return scene


CASES = {
    "heterogeneous 96": lambda: workloads.heterogeneous(96, spheres=40),
    "blocks and slabs": blocks_and_slabs,
    "graded": lambda: scenes.graded()[0],
    "materials": lambda: scenes.materials()[0],
    "mixed 1": lambda: workloads.mixed_scene(11, lo=33, hi=70),
    "mixed 2": lambda: workloads.mixed_scene(12, lo=33, hi=70),
    "300 materials (u16 index)": lambda: __import__("tests.test_setup_parity", fromlist=["x"]).many_materials(300, 26),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_device_raster_matches_the_oracle(case):
    scene = CASES[case]()
    resolved = ResolvedScene(scene)
    nx, ny, nz = resolved.extent
    dtype = np.uint8 if resolved.index_bytes == 1 else np.uint16
    expected = oracle.OracleSimulation(scene).table(_abi.DP_TABLE_MATERIAL_INDEX).astype(dtype)
    assert np.array_equal(resolved.table(_abi.DP_TABLE_MATERIAL_INDEX), expected)
    for pitch in (nx, (nx + 3) // 4 * 4, (nx + 15) // 16 * 16 + 16):
        rows = device_index(resolved, pitch)
        assert np.array_equal(rows[:, :nx].reshape(-1), expected), pitch
        assert not rows[:, nx:].any(), "padding bytes must be zero"
