"""dp_energy_noalloc: the energy reduction for callers that cannot allocate.

Some callers cannot call cudaMalloc where they need the field energy (it may
synchronize the device or fail, or their device memory belongs to another
allocator).  dp_energy_noalloc takes device pointers the caller already holds
and keeps its scratch in a fixed array inside the library.  Each case here
feeds it a simulation's own device fields (dp_sim_device_ptr, rows padded to
dp_sim_row_pitch cells) and checks it against dp_sim_energy on two calls in a
row.  This file runs last so that a failure here leaves every other test
already run; it must pass alone in a fresh process too.
"""
import ctypes as C

import numpy as np
import pytest

from diaphane_gb300 import _abi, Axis, Extent, Material, ResolvedScene, Scene, Shape, Simulation, Source, Waveform
from tests import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-9  # the energy tolerance the other device tests use


def device_tables(resolved: ResolvedScene):
    import torch
    scene = resolved.scene
    eps_mu = np.array([[m.relative_permittivity, m.relative_permeability] for m in scene.materials.materials],
                      np.float32).ravel()
    tables = {
        "material": torch.from_numpy(resolved.table(_abi.DP_TABLE_MATERIAL_INDEX).copy()).cuda(),
        "eps_mu": torch.from_numpy(eps_mu).cuda(),
        "materials": len(scene.materials.materials),
        "primary": torch.from_numpy(resolved.table(_abi.DP_TABLE_PRIMARY)).cuda(),
        "dual": torch.from_numpy(resolved.table(_abi.DP_TABLE_DUAL)).cuda(),
    }
    torch.cuda.synchronize()
    return tables


def stream_of(sim: Simulation) -> int:
    p = C.c_void_p()
    _abi.check(_abi.lib().dp_sim_stream(sim.handle, C.byref(p)))
    return p.value or 0


def noalloc_energy(sim: Simulation, resolved: ResolvedScene, t, out):
    lib = _abi.lib()
    extent = (C.c_uint32 * 3)(*resolved.extent)
    return lib.dp_energy_noalloc(sim.device_ptr(_abi.DP_FIELD_ELECTRIC), sim.device_ptr(_abi.DP_FIELD_MAGNETIC),
                                 lib.dp_sim_row_pitch(sim.handle), t["material"].data_ptr(), resolved.index_bytes, 0,
                                 t["eps_mu"].data_ptr(), t["materials"], t["primary"].data_ptr(),
                                 t["dual"].data_ptr(), extent, out.data_ptr(), stream_of(sim))


def check_two_calls(scene, steps: int, more: int = 7):
    import torch
    resolved = ResolvedScene(scene)
    sim = Simulation(resolved)
    sim.advance_by(steps)
    t = device_tables(resolved)
    out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    for call in range(2):
        expected = sim.energy()   # synchronizes the simulation's stream
        _abi.check(noalloc_energy(sim, resolved, t, out))
        sim.wait()
        got = out.cpu().numpy()
        assert expected.total() > 0
        assert abs(got[0] - expected.electric) <= RTOL * expected.electric, (call, got, expected)
        assert abs(got[1] - expected.magnetic) <= RTOL * expected.magnetic, (call, got, expected)
        sim.advance_by(more)  # the second call sees different fields
    return sim


def test_dense_rows():
    """44×40×40: rows of 44 cells are not padded; two reduction blocks."""
    scene, _ = scenes.materials()
    sim = check_two_calls(scene, 120)
    assert _abi.lib().dp_sim_row_pitch(sim.handle) == 44


def lossy_box(n):
    scene = Scene.empty(Extent(*n), 1e-3)
    frequency = scene.grid.frequency_for_resolution(16.0)
    glass = scene.materials.push(Material.refractive(1.7))
    lossy = scene.materials.push(Material.matched_lossy(2.0, 0.05))
    scene.shapes.append(Shape.sphere((4e-3, 0.0, 0.0), 9e-3, glass))
    scene.shapes.append(Shape.sphere((-12e-3, 3e-3, 0.0), 5e-3, lossy))
    scene.sources.append(Source.point((-2e-3, -4e-3, 1e-3), Axis.Z, Waveform.ricker(frequency)))
    return scene


@pytest.mark.parametrize("extent", [(45, 40, 40), (101, 90, 80)])
def test_padded_rows_and_many_blocks(extent):
    """nx % 4 != 0, so the simulation's rows are padded; 101×90×80 spans 12
    reduction blocks, the last one partial."""
    sim = check_two_calls(lossy_box(extent), 150)
    assert _abi.lib().dp_sim_row_pitch(sim.handle) == (extent[0] + 3) // 4 * 4 != extent[0]


def test_a_u16_index_past_256_materials():
    from tests.test_setup_parity import many_materials
    scene = many_materials(300, side=30)
    frequency = scene.grid.frequency_for_resolution(8.0)
    scene.sources.append(Source.point((0.0005, 0.0, 0.0), Axis.Z, Waveform.ricker(frequency)))
    assert ResolvedScene(scene).index_bytes == 2
    check_two_calls(scene, 60)


def test_an_index_past_the_material_count_gives_nan():
    import torch
    scene, _ = scenes.materials()
    resolved = ResolvedScene(scene)
    sim = Simulation(resolved)
    sim.advance_by(40)
    t = device_tables(resolved)
    t["materials"] = 2  # the scene uses 4; indices 2 and 3 are now out of range
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    _abi.check(noalloc_energy(sim, resolved, t, out))
    sim.wait()
    assert np.isnan(out.cpu().numpy()).all()


def test_grids_beyond_its_scratch_are_rejected():
    import torch
    small = torch.zeros(16, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    extent = (C.c_uint32 * 3)(1024, 1024, 512)  # 2^29 cells: over the 2^28 limit, rejected before any launch
    p = small.data_ptr()
    status = _abi.lib().dp_energy_noalloc(p, p, 0, p, 1, 0, p, 1, p, p, extent, out.data_ptr(), None)
    assert status == _abi.DP_ERR_RANGE
    assert b"2^28" in _abi.lib().dp_last_error()
    bad_width = _abi.lib().dp_energy_noalloc(p, p, 0, p, 3, 0, p, 1, p, p, (C.c_uint32 * 3)(4, 4, 4),
                                             out.data_ptr(), None)
    assert bad_width == _abi.DP_ERR_INVALID
