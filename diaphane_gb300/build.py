"""Builds the CUDA library in-tree: diaphane_gb300/libdiaphane_gb300.so.

nvcc compiles the kernels for sm_103a only; g++ compiles the host setup.  The
device code is built with -fmad=false (no multiply-add contraction) and the
host code with -ffp-contract=off, so both evaluate the update expressions in
the reference's f32 order.  Objects are compiled in parallel and cached by
source hash under diaphane_gb300/_build/.
"""
from __future__ import annotations

import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys
from pathlib import Path

PACKAGE = Path(__file__).resolve().parent
ROOT = PACKAGE.parent
CSRC = PACKAGE / "csrc"
BUILD = PACKAGE / "_build"
LIBRARY = PACKAGE / "libdiaphane_gb300.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-fmad=false", "-prec-div=true", "-prec-sqrt=true",
              "-ftz=false", "-Xcompiler", "-fPIC,-ffp-contract=off,-fopenmp", "-Xptxas", "-v"]
GXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fopenmp", "-Wall", "-Wextra"]


def _nvcc() -> str:
    for candidate in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if candidate and Path(candidate).exists():
            return candidate
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build diaphane_gb300")


def _digest(path: Path, flags: list[str]) -> str:
    h = hashlib.sha256()
    h.update(" ".join(flags).encode())
    h.update(path.read_bytes())
    for header in sorted(CSRC.glob("*.h*")) + sorted(CSRC.glob("*.cuh")) + [ROOT / "include" / "diaphane_gb300.h"]:
        h.update(header.read_bytes())
    return h.hexdigest()[:16]


def _compile(source: Path) -> tuple[Path, str]:
    if source.suffix == ".cu":
        flags = ARCH + NVCC_FLAGS
        compiler = [_nvcc()]
    else:
        flags = GXX_FLAGS
        compiler = [os.environ.get("CXX", "g++")]
    obj = BUILD / f"{source.stem}-{_digest(source, flags)}.o"
    log = ""
    if not obj.exists():
        cmd = compiler + flags + ["-I", str(ROOT / "include"), "-c", str(source), "-o", str(obj)]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        log = proc.stdout + proc.stderr
        if proc.returncode != 0:
            raise RuntimeError(f"compiling {source.name} failed:\n{' '.join(cmd)}\n{log}")
        (BUILD / f"{obj.stem}.log").write_text(log)
    return obj, log


def build(verbose: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    sources = sorted(CSRC.glob("*.cu")) + sorted(CSRC.glob("*.cpp"))
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, len(sources))) as pool:
        results = list(pool.map(_compile, sources))
    objects = [obj for obj, _ in results]
    if verbose:
        for _, log in results:
            if log:
                print(log, file=sys.stderr)
    stamp = BUILD / ("link-" + hashlib.sha256(" ".join(str(o) for o in objects).encode()).hexdigest()[:16])
    if not LIBRARY.exists() or not stamp.exists():
        tmp = LIBRARY.with_suffix(".so.tmp")
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objects] + ["-lgomp"]
        proc = subprocess.run(cmd, capture_output=True, text=True)
        if proc.returncode != 0:
            raise RuntimeError(f"linking failed:\n{' '.join(cmd)}\n{proc.stdout}{proc.stderr}")
        os.replace(tmp, LIBRARY)
        for old in BUILD.glob("link-*"):
            old.unlink()
        stamp.write_text("")
    return LIBRARY


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
