"""`bench.py --impl reference` on the CPU: the reference arm's one JSON line
keeps the benchmark contract (metric, unit, the warm-up asked for, a
cpu_baseline naming the port and its cores, an e2e with no host-device
bytes), on a small grid and a short budget; under torchrun only rank 0
prints."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def run(env_extra=None):
    env = dict(os.environ)
    env.update(env_extra or {})
    cmd = [sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--side", "32", "--steps", "4",
           "--warmup", "3", "--ref-budget", "2"]
    return subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=ROOT)


def test_reference_arm_prints_one_line_with_the_contract_keys():
    proc = run()
    assert proc.returncode == 0, proc.stderr[-2000:]
    lines = [l for l in proc.stdout.splitlines() if l.strip()]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference"
    assert line["metric"] == "Gcell-updates/s" and line["unit"] == "Gcell/s"
    assert line["higher_is_better"] is True and line["value"] > 0
    assert line["warmup"] == 3 and 1 <= line["steps"] <= 4
    assert line["config"]["workload"] == "heterogeneous scatterers 32^3"
    cpu = line["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == line["value"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_is_rank_zero_only():
    proc = run({"WORLD_SIZE": "2", "RANK": "1", "LOCAL_RANK": "1"})
    assert proc.returncode == 0, proc.stderr[-2000:]
    assert proc.stdout.strip() == ""


def test_reference_arm_loads_the_oracle_and_not_the_cuda_library():
    """The reference arm is the CPU restatement alone: its process maps
    oracle/liboracle.so and never the product's libdiaphane_gb300.so, not
    even to build the scene."""
    proc = run()
    assert proc.returncode == 0, proc.stderr[-2000:]
    line = json.loads([l for l in proc.stdout.splitlines() if l.strip()][0])
    loaded = line["libraries_loaded"]
    assert "oracle/liboracle.so" in loaded
    assert not any("libdiaphane_gb300" in name for name in loaded), loaded


def test_the_oracle_grid_resolver_matches_the_library():
    """Both resolvers give the same bits for every workload's grid, so the
    reference arm's scene is the one the CUDA arm steps."""
    import ctypes as C
    import oracle
    from diaphane_gb300 import _abi, workloads
    from diaphane_gb300.scene import LibraryGridResolver
    grids = [workloads.heterogeneous(64).grid, workloads.graded_stack().grid, workloads.graded_cavity().grid,
             workloads.free_flight(80).grid, workloads.mixed_scene(7).grid]
    for grid in grids:
        spec, keep = grid.spec()
        a, b = _abi.dp_grid_info(), _abi.dp_grid_info()
        LibraryGridResolver.resolve(spec, a)
        oracle.OracleGridResolver.resolve(spec, b)
        assert bytes(a) == bytes(b)
        for op in range(4):
            src = _abi.F3(0.001, -0.002, 0.0) if op in (0, 2) else _abi.F3(3.0, 4.0, 5.0)
            x, y = _abi.F3(), _abi.F3()
            LibraryGridResolver.map(spec, op, src, x)
            oracle.OracleGridResolver.map(spec, op, src, y)
            assert bytes(x) == bytes(y), (op, tuple(x), tuple(y))
        del keep
