"""dp_energy_noalloc: the energy reduction for callers that cannot allocate.

Some callers cannot call cudaMalloc where they need the field energy (it may
synchronize the device or fail, or their device memory belongs to another
allocator).  dp_energy_noalloc takes device pointers the caller already holds
and keeps its scratch in a fixed array inside the library.  This file runs
last so that a failure here leaves every other test already run; it must pass
alone in a fresh process too.
"""
import ctypes as C

import numpy as np
import pytest

from diaphane_gb300 import _abi, ResolvedScene, Simulation
from tests import scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-9  # the energy tolerance the other device tests use


def device_tables(resolved: ResolvedScene):
    import torch
    scene = resolved.scene
    eps_mu = np.array([[m.relative_permittivity, m.relative_permeability] for m in scene.materials.materials],
                      np.float32).ravel()
    tables = {
        "material": torch.from_numpy(resolved.table(_abi.DP_TABLE_MATERIAL_INDEX)).cuda(),
        "eps_mu": torch.from_numpy(eps_mu).cuda(),
        "primary": torch.from_numpy(resolved.table(_abi.DP_TABLE_PRIMARY)).cuda(),
        "dual": torch.from_numpy(resolved.table(_abi.DP_TABLE_DUAL)).cuda(),
    }
    torch.cuda.synchronize()
    return tables


def stream_of(sim: Simulation) -> int:
    p = C.c_void_p()
    _abi.check(_abi.lib().dp_sim_stream(sim.handle, C.byref(p)))
    return p.value or 0


def test_no_alloc_energy_matches_dp_sim_energy_on_two_calls_in_a_row():
    import torch
    scene, _ = scenes.materials()
    resolved = ResolvedScene(scene)
    sim = Simulation(resolved)
    sim.advance_by(120)
    t = device_tables(resolved)
    out = torch.full((2,), -1.0, dtype=torch.float64, device="cuda")
    extent = (C.c_uint32 * 3)(*resolved.extent)
    lib = _abi.lib()
    for call in range(2):
        expected = sim.energy()   # synchronizes the simulation's stream
        status = lib.dp_energy_noalloc(sim.device_ptr(_abi.DP_FIELD_ELECTRIC), sim.device_ptr(_abi.DP_FIELD_MAGNETIC),
                                       t["material"].data_ptr(), t["eps_mu"].data_ptr(), t["primary"].data_ptr(),
                                       t["dual"].data_ptr(), extent, out.data_ptr(), stream_of(sim))
        _abi.check(status)
        sim.wait()
        got = out.cpu().numpy()
        assert expected.total() > 0
        assert abs(got[0] - expected.electric) <= RTOL * expected.electric, (call, got, expected)
        assert abs(got[1] - expected.magnetic) <= RTOL * expected.magnetic, (call, got, expected)
        sim.advance_by(7)  # the second call sees different fields


def test_no_alloc_energy_rejects_grids_beyond_its_scratch():
    import torch
    small = torch.zeros(16, device="cuda")
    out = torch.zeros(2, dtype=torch.float64, device="cuda")
    extent = (C.c_uint32 * 3)(1024, 1024, 512)  # 2^29 cells: over the 2^28 limit, rejected before any launch
    p = small.data_ptr()
    status = _abi.lib().dp_energy_noalloc(p, p, p, p, p, p, extent, out.data_ptr(), None)
    assert status == 7  # DP_ERR_RANGE
    assert b"2^28" in _abi.lib().dp_last_error()
