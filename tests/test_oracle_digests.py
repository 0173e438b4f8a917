"""The oracle still produces the bits it was pinned with: every case of
tests/golden/oracle_digests.json re-run here, on a different thread count
than the one that wrote it (the sweeps over z planes leave each cell's
arithmetic unchanged, so the digest may not move)."""
import json
import platform
from pathlib import Path

import pytest

from tests.golden import make_oracle_digests as golden

TABLE = json.loads((Path(__file__).resolve().parent / "golden" / "oracle_digests.json").read_text())
CASES = {name: (scene, steps) for name, scene, steps in golden.cases()}


@pytest.mark.skipif(platform.machine() != TABLE["machine"], reason="digests were written on another architecture")
@pytest.mark.parametrize("name", sorted(TABLE["cases"]))
def test_oracle_reproduces_its_pinned_bits(name):
    scene, steps = CASES[name]
    assert steps == TABLE["cases"][name]["steps"]
    assert golden.digest(scene, steps, threads=1) == TABLE["cases"][name]["sha256"], name
