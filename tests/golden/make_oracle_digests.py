"""Writes oracle_digests.json: SHA-256 digests of the oracle's E, H and
intensity after a fixed number of steps on every shared parity scene and a
small heterogeneous scene.  The oracle was pinned against the reference's
known-answer and acceptance tests; these digests then hold it to the exact
bits it had at that point, so a change of source, compiler flags or thread
count that moves any bit of the checker fails the CPU suite.  The waveforms
call the platform's libm, so the digests hold for the machine architecture
recorded beside them.

    python tests/golden/make_oracle_digests.py
"""
from __future__ import annotations

import hashlib
import json
import platform
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
sys.path.insert(0, str(HERE.parent.parent))

STEPS = 60


def cases():
    from diaphane_gb300 import workloads
    from tests import scenes
    out = [("heterogeneous_48", workloads.heterogeneous(48), STEPS)]
    for name, make in scenes.PARITY_CASES.items():
        scene, steps = make()
        out.append((name, scene, min(steps, STEPS)))
    return out


def digest(scene, steps: int, threads: int) -> str:
    import oracle
    sim = oracle.OracleSimulation(scene, threads=threads)
    sim.set_accumulate_intensity(True)
    sim.advance_by(steps)
    h = hashlib.sha256()
    for part in (sim.read_electric(), sim.read_magnetic(), sim.read_intensity()):
        h.update(part.tobytes())
    return h.hexdigest()


def main() -> None:
    table = {name: {"steps": steps, "sha256": digest(scene, steps, threads=4)} for name, scene, steps in cases()}
    out = {"machine": platform.machine(), "cases": table}
    (HERE / "oracle_digests.json").write_text(json.dumps(out, indent=1, sort_keys=True) + "\n")
    print(f"{len(table)} digests written")


if __name__ == "__main__":
    main()
