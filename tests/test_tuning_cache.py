"""The tuned-plan cache's text form on the CPU: what import accepts and
rejects, what export gives back, and the buffer-size contract of the C
entry point.  (Tuning itself, and a later simulation starting from the tuned
plan, are GPU tests.)"""
import ctypes as C

import pytest

from diaphane_gb300 import _abi
from diaphane_gb300.simulation import tuning_cache_clear, tuning_cache_export, tuning_cache_import


@pytest.fixture(autouse=True)
def empty_cache():
    tuning_cache_clear()
    yield
    tuning_cache_clear()


def test_imported_lines_come_back_from_export():
    assert tuning_cache_export() == ""
    tuning_cache_import("512 512 512 152 4 8 3 27 1.426\n\n96 80 64 152 2 8 3 24 0.02\n")
    lines = tuning_cache_export().splitlines()
    assert lines == ["96 80 64 152 2 8 3 24 0.02", "512 512 512 152 4 8 3 27 1.426"]
    # A second import of the same shape replaces its plan.
    tuning_cache_import("96 80 64 152 1 8 4 16 0.03")
    assert tuning_cache_export().splitlines()[0] == "96 80 64 152 1 8 4 16 0.03"
    tuning_cache_clear()
    assert tuning_cache_export() == ""


@pytest.mark.parametrize("line", ["512 512 512 152 4 8 3 27",          # a field short
                                  "512 512 512 152 4 8 3 27 1.0 9",    # one too many
                                  "512 512 512 152 3 8 3 27 1.0",      # no such tile shape
                                  "512 512 512 152 4 8 3 600 1.0",     # deeper than the grid
                                  "0 512 512 152 4 8 3 16 1.0",        # empty grid
                                  "a b c"])
def test_a_malformed_line_is_refused_and_the_lines_before_it_kept(line):
    with pytest.raises(_abi.DiaphaneError) as err:
        tuning_cache_import("64 64 64 152 2 8 3 16 0.01\n" + line + "\n")
    assert err.value.status == _abi.DP_ERR_INVALID
    assert tuning_cache_export() == "64 64 64 152 2 8 3 16 0.01\n"


def test_export_reports_the_length_it_needs():
    tuning_cache_import("64 64 64 152 2 8 3 16 0.01")
    need = C.c_size_t()
    small = C.create_string_buffer(8)
    assert _abi.lib().dp_tune_cache_export(small, len(small), C.byref(need)) == _abi.DP_ERR_RANGE
    assert need.value == len("64 64 64 152 2 8 3 16 0.01\n")
    big = C.create_string_buffer(need.value + 1)
    assert _abi.lib().dp_tune_cache_export(big, len(big), C.byref(need)) == _abi.DP_OK
    assert big.value.decode() == "64 64 64 152 2 8 3 16 0.01\n"
