"""ORACLE — test infrastructure only.

ctypes binding of oracle/liboracle.so, the CPU restatement of the reference
solver (kvark/diaphane src/cpu.rs and its setup in src/grid.rs,
src/material.rs, src/boundary.rs, src/source.rs, src/scene.rs).  Imported by
tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs only; the
product never loads it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from diaphane_gb300 import _abi
from diaphane_gb300.scene import Scene

from .build import LIBRARY, build

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        build()
        h = C.CDLL(str(LIBRARY))
        P = C.c_void_p
        sigs = {
            "or_last_error": (C.c_char_p, []),
            "or_sim_create": (C.c_int, [C.POINTER(_abi.dp_scene_desc), C.c_int, C.POINTER(P)]),
            "or_sim_destroy": (None, [P]),
            "or_sim_set_threads": (None, [P, C.c_int]),
            "or_sim_advance": (C.c_int, [P, C.c_uint64]),
            "or_sim_reverse": (C.c_int, [P, C.c_uint64]),
            "or_sim_reset": (None, [P]),
            "or_sim_step_count": (C.c_uint64, [P]),
            "or_sim_time": (C.c_float, [P]),
            "or_sim_is_reversible": (C.c_int, [P]),
            "or_sim_set_accumulate_intensity": (None, [P, C.c_int]),
            "or_sim_accumulated_steps": (C.c_uint64, [P]),
            "or_sim_read_field": (C.c_int, [P, C.c_int, P]),
            "or_sim_read_field64": (C.c_int, [P, C.c_int, P]),
            "or_sim_write_field": (C.c_int, [P, C.c_int, P]),
            "or_sim_restore": (C.c_int, [P, C.c_uint64, P, P]),
            "or_sim_sample": (C.c_float, [P, C.c_int, C.c_int, C.c_uint32, C.c_uint32, C.c_uint32]),
            "or_sim_component": (C.c_int, [P, C.c_int, C.c_int, P]),
            "or_sim_energy": (None, [P, C.POINTER(C.c_double), C.POINTER(C.c_double)]),
            "or_sim_energy_density": (C.c_int, [P, P]),
            "or_sim_is_finite": (C.c_int, [P]),
            "or_sim_extent": (None, [P, C.POINTER(C.c_uint32)]),
            "or_sim_time_step": (C.c_float, [P]),
            "or_sim_table": (C.c_int, [P, C.c_int, P]),
            "or_sim_absorber_peak": (C.c_float, [P]),
            "or_sim_injections": (C.c_int, [P, C.c_float, C.POINTER(_abi.dp_injection), C.c_uint32,
                                            C.POINTER(C.c_uint32)]),
            "or_injection_weight": (C.c_float, [C.POINTER(_abi.dp_injection), C.POINTER(C.c_float)]),
            "or_grid_resolve": (C.c_int, [C.POINTER(_abi.dp_grid_spec), C.POINTER(C.c_uint32), C.POINTER(C.c_float),
                                          C.POINTER(C.c_float), C.POINTER(C.c_float), C.POINTER(C.c_float),
                                          C.POINTER(C.c_float)]),
            "or_grid_info": (C.c_int, [C.POINTER(_abi.dp_grid_spec), C.POINTER(_abi.dp_grid_info)]),
            "or_grid_map": (C.c_int, [C.POINTER(_abi.dp_grid_spec), C.c_int, C.POINTER(C.c_float),
                                      C.POINTER(C.c_float)]),
            "or_numerical_phase_velocity": (C.c_float, [C.c_float, C.c_float, C.POINTER(C.c_float)]),
            "or_waveform_evaluate": (C.c_float, [C.POINTER(_abi.dp_waveform), C.c_float]),
            "or_max_threads": (C.c_int, []),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(h, name)
            fn.restype = res
            fn.argtypes = args
        _lib = h
    return _lib


class OracleError(RuntimeError):
    pass


def _check(rc: int) -> None:
    if rc != 0:
        raise OracleError(lib().or_last_error().decode(errors="replace"))


class OracleSimulation:
    """cpu::Simulation (src/cpu.rs:65-713), restated.  fp64=True is the FP64 run."""

    def __init__(self, scene: Scene, fp64: bool = False, threads: int = 1):
        self.scene = scene
        desc, keep = scene.desc()
        h = C.c_void_p()
        _check(lib().or_sim_create(C.byref(desc), int(fp64), C.byref(h)))
        del keep
        self.handle = h
        self.fp64 = fp64
        ext = (C.c_uint32 * 3)()
        lib().or_sim_extent(self.handle, ext)
        self.extent = tuple(ext)
        self.cells = int(np.prod(self.extent))
        self.set_threads(threads)

    def __del__(self):
        if getattr(self, "handle", None):
            lib().or_sim_destroy(self.handle)
            self.handle = None

    def set_threads(self, threads: int) -> None:
        lib().or_sim_set_threads(self.handle, max(1, int(threads)))

    def advance(self) -> None:
        self.advance_by(1)

    def advance_by(self, steps: int) -> None:
        _check(lib().or_sim_advance(self.handle, steps))

    def reverse(self) -> None:
        self.reverse_by(1)

    def reverse_by(self, steps: int) -> None:
        _check(lib().or_sim_reverse(self.handle, steps))

    def reset(self) -> None:
        lib().or_sim_reset(self.handle)

    def step_count(self) -> int:
        return lib().or_sim_step_count(self.handle)

    def time(self) -> float:
        return lib().or_sim_time(self.handle)

    def time_step(self) -> float:
        return lib().or_sim_time_step(self.handle)

    def is_reversible(self) -> bool:
        return bool(lib().or_sim_is_reversible(self.handle))

    def set_accumulate_intensity(self, on: bool) -> None:
        lib().or_sim_set_accumulate_intensity(self.handle, int(on))

    def accumulated_steps(self) -> int:
        return lib().or_sim_accumulated_steps(self.handle)

    def _read(self, field: int, count: int, fp64: bool) -> np.ndarray:
        out = np.empty(count, dtype=np.float64 if fp64 else np.float32)
        fn = lib().or_sim_read_field64 if fp64 else lib().or_sim_read_field
        _check(fn(self.handle, field, out.ctypes.data))
        return out

    def read_electric(self, fp64: bool = False) -> np.ndarray:
        return self._read(_abi.DP_FIELD_ELECTRIC, 3 * self.cells, fp64)

    def read_magnetic(self, fp64: bool = False) -> np.ndarray:
        return self._read(_abi.DP_FIELD_MAGNETIC, 3 * self.cells, fp64)

    def read_intensity(self, fp64: bool = False) -> np.ndarray:
        return self._read(_abi.DP_FIELD_INTENSITY, self.cells, fp64)

    def _component(self, field: int, axis: int) -> np.ndarray:
        out = np.empty(self.cells, dtype=np.float32)
        _check(lib().or_sim_component(self.handle, field, int(axis), out.ctypes.data))
        return out

    def electric(self, axis: int) -> np.ndarray:
        return self._component(_abi.DP_FIELD_ELECTRIC, axis)

    def magnetic(self, axis: int) -> np.ndarray:
        return self._component(_abi.DP_FIELD_MAGNETIC, axis)

    def sample_electric(self, axis: int, coord) -> float:
        return lib().or_sim_sample(self.handle, _abi.DP_FIELD_ELECTRIC, int(axis), *[int(c) for c in coord])

    def sample_magnetic(self, axis: int, coord) -> float:
        return lib().or_sim_sample(self.handle, _abi.DP_FIELD_MAGNETIC, int(axis), *[int(c) for c in coord])

    def index(self, coord) -> int:
        return (coord[2] * self.extent[1] + coord[1]) * self.extent[0] + coord[0]

    def write_electric(self, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float32)
        _check(lib().or_sim_write_field(self.handle, _abi.DP_FIELD_ELECTRIC, v.ctypes.data))

    def write_magnetic(self, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float32)
        _check(lib().or_sim_write_field(self.handle, _abi.DP_FIELD_MAGNETIC, v.ctypes.data))

    def energy(self):
        from diaphane_gb300.simulation import Energy
        e, m = C.c_double(), C.c_double()
        lib().or_sim_energy(self.handle, C.byref(e), C.byref(m))
        return Energy(e.value, m.value)

    def energy_density(self) -> np.ndarray:
        out = np.empty(self.cells, dtype=np.float32)
        _check(lib().or_sim_energy_density(self.handle, out.ctypes.data))
        return out

    def is_finite(self) -> bool:
        return bool(lib().or_sim_is_finite(self.handle))

    def absorber_peak(self) -> float:
        return lib().or_sim_absorber_peak(self.handle)

    def table(self, which: int) -> np.ndarray:
        span = sum(self.extent)
        sizes = {
            _abi.DP_TABLE_MAGNETIC_GAINS: (span, np.float32),
            _abi.DP_TABLE_ELECTRIC_GAINS: (span, np.float32),
            _abi.DP_TABLE_CELL_CENTERS: (span, np.float32),
            _abi.DP_TABLE_ABSORBER: (2 * span, np.float32),
            _abi.DP_TABLE_COEFFICIENTS: (4 * len(self.scene.materials), np.float32),
            _abi.DP_TABLE_MATERIAL_INDEX: (self.cells, np.uint32),
            _abi.DP_TABLE_PRIMARY: (span, np.float32),
            _abi.DP_TABLE_DUAL: (span, np.float32),
        }
        count, dtype = sizes[which]
        out = np.empty(count, dtype=dtype)
        _check(lib().or_sim_table(self.handle, which, out.ctypes.data))
        return out

    def injections(self, time: float) -> list:
        capacity = 2 * max(1, len(self.scene.sources))
        buf = (_abi.dp_injection * capacity)()
        count = C.c_uint32()
        _check(lib().or_sim_injections(self.handle, time, buf, capacity, C.byref(count)))
        return [buf[i] for i in range(count.value)]

    # Steppable
    def snapshot(self):
        from diaphane_gb300.simulation import Snapshot
        return Snapshot(self.step_count(), self.read_electric(), self.read_magnetic())

    def restore(self, snapshot) -> None:
        e = np.ascontiguousarray(snapshot.electric, dtype=np.float32)
        h = np.ascontiguousarray(snapshot.magnetic, dtype=np.float32)
        _check(lib().or_sim_restore(self.handle, snapshot.step, e.ctypes.data, h.ctypes.data))


def injection_weight(injection, position) -> float:
    return lib().or_injection_weight(C.byref(injection), (C.c_float * 3)(*position))


def numerical_phase_velocity(courant: float, cells: float, direction) -> float:
    return lib().or_numerical_phase_velocity(courant, cells, (C.c_float * 3)(*direction))


def waveform_evaluate(waveform, time: float) -> float:
    w = waveform.to_c()
    return lib().or_waveform_evaluate(C.byref(w), time)


def grid_resolve(grid):
    spec, keep = grid.spec()
    ext = (C.c_uint32 * 3)()
    size = (C.c_float * 3)()
    dt, worst, finest, coarsest = C.c_float(), C.c_float(), C.c_float(), C.c_float()
    _check(lib().or_grid_resolve(C.byref(spec), ext, C.byref(dt), C.byref(worst), C.byref(finest),
                                 C.byref(coarsest), size))
    del keep
    return {"extent": tuple(ext), "time_step": dt.value, "worst_ratio": worst.value, "finest": finest.value,
            "coarsest": coarsest.value, "size": tuple(size)}


def grid_map(grid, op: int, values) -> tuple:
    spec, keep = grid.spec()
    out = (C.c_float * 3)()
    _check(lib().or_grid_map(C.byref(spec), op, (C.c_float * 3)(*values), out))
    del keep
    return tuple(out)


class OracleGridResolver:
    """Grid recipes resolved by the oracle's own restatement of Grid::build
    (src/grid.rs:466-594, 695-745), for scene.use_grid_resolver: a process
    that times the CPU baseline builds its scenes without loading the CUDA
    library."""

    @staticmethod
    def resolve(spec, out) -> None:
        _check(lib().or_grid_info(C.byref(spec), C.byref(out)))

    @staticmethod
    def map(spec, op: int, src, dst) -> None:
        _check(lib().or_grid_map(C.byref(spec), op, src, dst))


def max_threads() -> int:
    return lib().or_max_threads()
