"""The step kernel's division wrapper against the library's IEEE division.

The fused step divides by (1 + loss) through a wrapper that avoids the slow
path for zero and tiny numerators; it must agree with n / d bit for bit for
every numerator class and the divisors the updates use (d = 1 + loss >= 1).
"""
import ctypes as C

import numpy as np
import pytest

from diaphane_gb300 import _abi

pytestmark = pytest.mark.gpu


def run(n: np.ndarray, d: np.ndarray):
    fn = _abi.lib().dp_internal_division_check
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p] * 4 + [C.c_size_t]
    n = np.ascontiguousarray(n, np.float32)
    d = np.ascontiguousarray(d, np.float32)
    ours, ieee = np.empty_like(n), np.empty_like(n)
    assert fn(n.ctypes.data, d.ctypes.data, ours.ctypes.data, ieee.ctypes.data, n.size) == 0
    return ours, ieee


def test_random_numerators_of_every_magnitude():
    rng = np.random.default_rng(11)
    count = 1 << 22
    sign = rng.choice([-1.0, 1.0], count)
    exponent = rng.uniform(-160, 10, count)
    n = (sign * rng.uniform(1, 2, count) * 2.0 ** exponent).astype(np.float32)
    d = (1.0 + rng.uniform(0, 4, count) ** rng.uniform(0.2, 3, count)).astype(np.float32)
    ours, ieee = run(n, d)
    assert np.array_equal(ours.view(np.uint32), ieee.view(np.uint32))


def test_edge_cases():
    tiny = np.array([0.0, -0.0, 1e-45, -1e-45, 2e-45, 3e-45, 1e-40, -1e-40, 1.1754942e-38, 1.1754944e-38,
                     2 ** -100, -(2 ** -100), 2 ** -101, 7.0e-31, np.inf, -np.inf, 1.0, -1.0, 3.4e38], np.float32)
    divisors = np.array([1.0, 1.0000001, 1.5, 2.0, 2.9999998, 3.0, 3.3333333, 4.2, 17.0], np.float32)
    n = np.repeat(tiny, divisors.size)
    d = np.tile(divisors, tiny.size)
    ours, ieee = run(n, d)
    assert np.array_equal(ours.view(np.uint32), ieee.view(np.uint32))
    # Subnormal quotients that sit exactly on rounding midpoints of the grid.
    k = np.arange(1, 1 << 16, dtype=np.float64)
    n = (k * 2.0 ** -149 * 3.0).astype(np.float32)
    ours, ieee = run(n, np.full(n.size, 2.0, np.float32))
    assert np.array_equal(ours.view(np.uint32), ieee.view(np.uint32))
    ours, ieee = run(-n, np.full(n.size, 6.0, np.float32))
    assert np.array_equal(ours.view(np.uint32), ieee.view(np.uint32))
