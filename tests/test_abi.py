"""The C ABI library loads on a machine without a GPU and exports every entry
point include/diaphane_gb300.h declares; no compute call is made here."""
import ctypes
import re
from pathlib import Path

from diaphane_gb300 import _abi

HEADER = Path(__file__).resolve().parent.parent / "include" / "diaphane_gb300.h"


def declared_functions():
    text = re.sub(r"/\*.*?\*/", "", HEADER.read_text(), flags=re.S)
    return sorted(set(re.findall(r"\b(dp_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_abi():
    names = declared_functions()
    assert "dp_sim_create" in names and "dp_sim_advance" in names and "dp_scene_create" in names
    assert len(names) >= 30


def test_library_exports_every_declared_symbol():
    lib = ctypes.CDLL(str(_abi.LIBRARY))
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, f"not exported: {missing}"


def test_python_binding_covers_every_declared_symbol():
    bound = {name for name, _, _ in _abi.SIGNATURES}
    assert set(declared_functions()) <= bound


def test_status_strings_and_errors():
    lib = _abi.lib()
    assert lib.dp_status_string(0) == b"ok"
    assert lib.dp_status_string(2).startswith(b"scene is lossy")
    # A null scene is rejected with a status, not a crash.
    status = lib.dp_scene_create(None, None)
    assert status == 1 and b"null" in lib.dp_last_error()


def test_read_buffers_are_checked_before_any_copy():
    import numpy as np
    import pytest
    from diaphane_gb300.simulation import _output
    assert _output(None, 5).shape == (5,)
    buf = np.zeros((2, 4), dtype=np.float32)
    view = _output(buf, 6)
    assert view.shape == (6,) and np.shares_memory(view, buf)
    for bad in [np.zeros(5, dtype=np.float64), np.zeros(4, dtype=np.float32), np.zeros((4, 4), np.float32)[:, 0]]:
        with pytest.raises(ValueError):
            _output(bad, 5)


def test_batch_bytes_saturate_instead_of_wrapping():
    """A probe series of probe_count x steps x 2 values is sized with an
    overflow check: past 2^40 values the scene's arena size reads UINT64_MAX
    (and dp_batch_add refuses it) rather than a wrapped small number.
    Host-only: no device call."""
    from diaphane_gb300 import Batch, Extent, ResolvedScene, Scene
    resolved = ResolvedScene(Scene.photon(Extent.cube(32)))
    plain = Batch.bytes_for(resolved, 100)
    assert 0 < plain < 1 << 30
    assert Batch.bytes_for(resolved, 100, probe_count=8) > plain
    assert Batch.bytes_for(resolved, 1 << 62, probe_count=8) == (1 << 64) - 1
    assert Batch.bytes_for(resolved, (1 << 40) // 16, probe_count=8) < 1 << 45
    assert Batch.bytes_for(resolved, 1 << 62, probe_count=0) < 1 << 30


def test_header_compiles_as_plain_c_and_cpp(tmp_path):
    """The boundary is a C ABI: the header must parse as pedantic C99 (what
    bindgen or cgo read) as well as C++."""
    import shutil
    import subprocess
    import pytest
    for compiler, std, suffix in (("gcc", "-std=c99", "c"), ("g++", "-std=c++11", "cpp")):
        if shutil.which(compiler) is None:
            pytest.skip(f"{compiler} not installed")
        src = tmp_path / f"h.{suffix}"
        src.write_text('#include "diaphane_gb300.h"\nint main(void) { return 0; }\n')
        proc = subprocess.run([compiler, std, "-Wall", "-Wextra", "-pedantic", "-Werror", "-fsyntax-only",
                               "-I", str(HEADER.parent), str(src)], capture_output=True, text=True)
        assert proc.returncode == 0, proc.stderr
