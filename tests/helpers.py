"""Shared comparison helpers, following the reference's parity harness
(tests/parity.rs:30-86): disagreement scaled by the peak over all three
components, with a guard against comparing an absorbed remnant."""
from __future__ import annotations

import numpy as np


def peak_of(values: np.ndarray) -> float:
    return float(np.max(np.abs(values))) if values.size else 0.0


def field_parity(reference: np.ndarray, candidate: np.ndarray, cells: int) -> tuple[float, float]:
    """(worst |Δ| over components / all-component peak, peak)."""
    assert reference.shape == candidate.shape == (3 * cells,)
    peak = peak_of(reference)
    worst = 0.0
    for a in range(3):
        r = reference[a * cells:(a + 1) * cells].astype(np.float64)
        c = candidate[a * cells:(a + 1) * cells].astype(np.float64)
        worst = max(worst, float(np.max(np.abs(r - c))))
    return (worst / peak if peak > 0 else float("inf")), peak


def assert_field_parity(name: str, reference: np.ndarray, candidate: np.ndarray, cells: int, steps: int,
                        tolerance: float) -> float:
    relative, peak = field_parity(reference, candidate, cells)
    assert peak > 0.0, f"{name} is identically zero after {steps} steps"
    assert peak > 2e-3, f"{name} peak {peak:e} after {steps} steps is an absorbed remnant"
    assert relative < tolerance, f"{name} diverged by {relative:e} of the {peak:e} peak after {steps} steps"
    return relative
