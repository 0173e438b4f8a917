"""Builds the oracle (test infrastructure) into oracle/liboracle.so.

g++ with -ffp-contract=off and no fast-math: the f32 instance evaluates the
reference's expressions in the reference's order.  OpenMP parallelizes the
sweeps over z planes only, which leaves every cell's arithmetic unchanged.
-O3, the optimization level of the reference's own release build (Cargo's
release profile), so that the timed CPU baseline is not handicapped; it
vectorizes loops without changing any result.
"""
from __future__ import annotations

import hashlib
import os
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SOURCE = HERE / "oracle.cpp"
LIBRARY = HERE / "liboracle.so"
FLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp", "-Wall", "-Wextra"]


def build() -> Path:
    digest = hashlib.sha256(SOURCE.read_bytes() + (ROOT / "include" / "diaphane_gb300.h").read_bytes()
                            + " ".join(FLAGS).encode()).hexdigest()[:16]
    stamp = HERE / f".liboracle-{digest}"
    if LIBRARY.exists() and stamp.exists():
        return LIBRARY
    tmp = LIBRARY.with_suffix(".so.tmp")
    cmd = [os.environ.get("CXX", "g++")] + FLAGS + ["-I", str(ROOT / "include"), str(SOURCE), "-o", str(tmp)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"building the oracle failed:\n{' '.join(cmd)}\n{proc.stdout}{proc.stderr}")
    os.replace(tmp, LIBRARY)
    for old in HERE.glob(".liboracle-*"):
        old.unlink()
    stamp.write_text("")
    return LIBRARY


if __name__ == "__main__":
    print(build())
