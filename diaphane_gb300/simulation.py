"""The simulation API of the reference's solvers, over the CUDA library.

``Simulation`` mirrors ``gpu::Simulation`` (src/gpu.rs:159-763) and the parts
of ``cpu::Simulation`` (src/cpu.rs:97-714) the two share: ``advance_by``,
``reverse_by``, ``reset``, ``read_electric``/``read_magnetic``/
``read_intensity``, ``component``, ``set_accumulate_intensity``,
``energy``, ``is_finite`` and the ``Steppable`` pair ``snapshot``/``restore``
(src/timeline.rs:63-72).  Every call goes through the C ABI; there is no CPU
path behind it.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import numpy as np

from . import _abi
from .scene import Axis, Scene


def _output(out, count: int) -> np.ndarray:
    """`out` (a contiguous float32 array of at least `count` values, e.g. a view
    of pinned host memory, which a copy reaches at full link speed) or a new
    array."""
    if out is None:
        return np.empty(count, dtype=np.float32)
    if out.dtype != np.float32 or not out.flags.c_contiguous or out.size < count:
        raise ValueError(f"out must be a contiguous float32 array of at least {count} values")
    return out.reshape(-1)[:count]


@dataclass
class Energy:
    """src/cpu.rs:52-62."""
    electric: float
    magnetic: float

    def total(self) -> float:
        return self.electric + self.magnetic


@dataclass
class Snapshot:
    """src/timeline.rs:43-55."""
    step: int
    electric: np.ndarray
    magnetic: np.ndarray

    def bytes(self) -> int:
        return self.electric.nbytes + self.magnetic.nbytes


class ResolvedScene:
    """The host-side setup of a scene (dp_scene): tables and injections."""

    def __init__(self, scene: Scene):
        self.scene = scene
        desc, keep = scene.desc()
        handle = C.c_void_p()
        _abi.check(_abi.lib().dp_scene_create(C.byref(desc), C.byref(handle)))
        del keep
        self.handle = handle
        info = _abi.dp_scene_info()
        _abi.check(_abi.lib().dp_scene_info_get(self.handle, C.byref(info)))
        self.extent = tuple(info.extent)
        self.cells = int(np.prod(self.extent))
        self.time_step = info.time_step
        self.absorber_peak = info.absorber_peak
        self.reversible = bool(info.reversible)
        self.material_count = info.material_count
        self.index_bytes = info.index_bytes

    def __del__(self):
        if getattr(self, "handle", None):
            _abi.lib().dp_scene_destroy(self.handle)
            self.handle = None

    def rasterize(self, device_ptr: int, row_pitch: int = 0, stream: int = 0) -> None:
        """The material index rasterized on the GPU into device memory at
        `device_ptr` (index_bytes per cell, rows of `row_pitch` cells, 0 = nx),
        on `stream`."""
        _abi.check(_abi.lib().dp_scene_raster(self.handle, C.c_void_p(device_ptr), row_pitch, C.c_void_p(stream)))

    def lookup_samples(self) -> int:
        return _abi.lib().dp_scene_lookup_samples(self.handle)

    def cell_lookup(self, samples: int = 0) -> np.ndarray:
        """Grid::cell_lookup: world-to-cell map, three sections of `samples`."""
        samples = samples or self.lookup_samples()
        out = np.empty(3 * samples, np.float32)
        _abi.check(_abi.lib().dp_scene_cell_lookup(self.handle, samples, out.ctypes.data, out.size))
        return out

    def table(self, which: int) -> np.ndarray:
        span = sum(self.extent)
        sizes = {
            _abi.DP_TABLE_MAGNETIC_GAINS: (span, np.float32),
            _abi.DP_TABLE_ELECTRIC_GAINS: (span, np.float32),
            _abi.DP_TABLE_CELL_CENTERS: (span, np.float32),
            _abi.DP_TABLE_ABSORBER: (2 * span, np.float32),
            _abi.DP_TABLE_COEFFICIENTS: (4 * self.material_count, np.float32),
            _abi.DP_TABLE_MATERIAL_INDEX: (self.cells, np.uint8 if self.index_bytes == 1 else np.uint16),
            _abi.DP_TABLE_PRIMARY: (span, np.float32),
            _abi.DP_TABLE_DUAL: (span, np.float32),
        }
        count, dtype = sizes[which]
        out = np.empty(count, dtype=dtype)
        _abi.check(_abi.lib().dp_scene_table(self.handle, which, out.ctypes.data, out.nbytes))
        return out

    def injections(self, time: float) -> list[_abi.dp_injection]:
        capacity = 2 * max(1, len(self.scene.sources))
        buf = (_abi.dp_injection * capacity)()
        count = C.c_uint32()
        _abi.check(_abi.lib().dp_scene_injections(self.handle, time, buf, capacity, C.byref(count)))
        return [buf[i] for i in range(count.value)]


class Simulation:
    """gpu::Simulation over the C ABI (one CUDA stream per handle)."""

    def __init__(self, scene: Scene | ResolvedScene, kernel: int = _abi.DP_KERNEL_AUTO, device: int = 0,
                 tile_y: int = 0, z_chunk: int = 0, cells_per_lane: int = 0, ring_slots: int = 0):
        self.resolved = scene if isinstance(scene, ResolvedScene) else ResolvedScene(scene)
        self.scene = self.resolved.scene
        opts = _abi.dp_options(device, kernel, tile_y, z_chunk, cells_per_lane, ring_slots)
        handle = C.c_void_p()
        _abi.check(_abi.lib().dp_sim_create(self.resolved.handle, C.byref(opts), C.byref(handle)))
        self.handle = handle
        self.extent = self.resolved.extent
        self.cells = self.resolved.cells

    def __del__(self):
        if getattr(self, "handle", None):
            _abi.lib().dp_sim_destroy(self.handle)
            self.handle = None

    def close(self) -> None:
        self.__del__()

    # -- stepping ---------------------------------------------------------------
    def advance(self) -> None:
        self.advance_by(1)

    def advance_by(self, steps: int) -> None:
        _abi.check(_abi.lib().dp_sim_advance(self.handle, steps))

    def reverse(self) -> None:
        self.reverse_by(1)

    def reverse_by(self, steps: int) -> None:
        _abi.check(_abi.lib().dp_sim_reverse(self.handle, steps))

    def reset(self) -> None:
        _abi.check(_abi.lib().dp_sim_reset(self.handle))

    def wait(self, timeout_ms: int = 120_000) -> None:
        _abi.check(_abi.lib().dp_sim_wait(self.handle, timeout_ms))

    def step_count(self) -> int:
        return _abi.lib().dp_sim_step_count(self.handle)

    def time(self) -> float:
        return _abi.lib().dp_sim_time(self.handle)

    def is_reversible(self) -> bool:
        return bool(_abi.lib().dp_sim_is_reversible(self.handle))

    @property
    def kernel(self) -> int:
        return _abi.lib().dp_sim_kernel(self.handle)

    def launch_count(self) -> int:
        return _abi.lib().dp_sim_launch_count(self.handle)

    # -- fields -----------------------------------------------------------------
    def _read(self, field: int, count: int, out=None) -> np.ndarray:
        out = _output(out, count)
        _abi.check(_abi.lib().dp_sim_read_field(self.handle, field, out.ctypes.data, count))
        return out

    def read_electric(self, out=None) -> np.ndarray:
        return self._read(_abi.DP_FIELD_ELECTRIC, 3 * self.cells, out)

    def read_magnetic(self, out=None) -> np.ndarray:
        return self._read(_abi.DP_FIELD_MAGNETIC, 3 * self.cells, out)

    def read_intensity(self, out=None) -> np.ndarray:
        return self._read(_abi.DP_FIELD_INTENSITY, self.cells, out)

    def component(self, values: np.ndarray, axis: Axis) -> np.ndarray:
        a = int(axis)
        return values[a * self.cells:(a + 1) * self.cells]

    def write_electric(self, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float32)
        _abi.check(_abi.lib().dp_sim_write_field(self.handle, _abi.DP_FIELD_ELECTRIC, v.ctypes.data, v.size))

    def write_magnetic(self, values: np.ndarray) -> None:
        v = np.ascontiguousarray(values, dtype=np.float32)
        _abi.check(_abi.lib().dp_sim_write_field(self.handle, _abi.DP_FIELD_MAGNETIC, v.ctypes.data, v.size))

    def device_ptr(self, field: int) -> int:
        p = C.c_void_p()
        _abi.check(_abi.lib().dp_sim_device_ptr(self.handle, field, C.byref(p)))
        return p.value

    def set_accumulate_intensity(self, on: bool) -> None:
        _abi.check(_abi.lib().dp_sim_set_accumulate_intensity(self.handle, int(on)))

    def accumulated_steps(self) -> int:
        return _abi.lib().dp_sim_accumulated_steps(self.handle)

    def bytes_per_step(self) -> int:
        return _abi.lib().dp_sim_bytes_per_step(self.handle)

    def field_bytes(self) -> int:
        return _abi.lib().dp_sim_field_bytes(self.handle)

    def energy(self) -> Energy:
        e, m = C.c_double(), C.c_double()
        _abi.check(_abi.lib().dp_sim_energy(self.handle, C.byref(e), C.byref(m)))
        return Energy(e.value, m.value)

    def energy_density(self) -> np.ndarray:
        out = np.empty(self.cells, np.float32)
        _abi.check(_abi.lib().dp_sim_energy_density(self.handle, out.ctypes.data, out.size))
        return out

    def _sample(self, field: int, axis: int, coord) -> float:
        c = (C.c_uint32 * 3)(*[int(v) for v in coord])
        out = C.c_float()
        _abi.check(_abi.lib().dp_sim_sample(self.handle, field, int(axis), c, C.byref(out)))
        return out.value

    def sample_electric(self, axis: Axis, coord) -> float:
        return self._sample(_abi.DP_FIELD_ELECTRIC, axis, coord)

    def sample_magnetic(self, axis: Axis, coord) -> float:
        return self._sample(_abi.DP_FIELD_MAGNETIC, axis, coord)

    def is_finite(self) -> bool:
        flag = C.c_int32()
        _abi.check(_abi.lib().dp_sim_is_finite(self.handle, C.byref(flag)))
        return bool(flag.value)

    # -- Steppable (src/timeline.rs:63-72) -----------------------------------------
    def snapshot(self) -> Snapshot:
        return Snapshot(self.step_count(), self.read_electric(), self.read_magnetic())

    def autotune(self, steps: int = 8) -> dict:
        """Times each fused-step plan from the current state and keeps the
        fastest; the state is restored exactly."""
        t = _abi.dp_tuning()
        _abi.check(_abi.lib().dp_sim_autotune(self.handle, steps, C.byref(t)))
        return {"cells_per_lane": t.cells_per_lane, "tile_y": t.tile_y, "ring_slots": t.ring_slots,
                "z_chunk": t.z_chunk, "ms_per_step": t.ms_per_step, "candidates": t.candidates}

    def plan(self) -> dict:
        """The fused-step plan the handle runs (all 0 on the
        one-thread-per-cell path)."""
        t = _abi.dp_tuning()
        _abi.check(_abi.lib().dp_sim_plan(self.handle, C.byref(t)))
        return {"cells_per_lane": t.cells_per_lane, "tile_y": t.tile_y, "ring_slots": t.ring_slots,
                "z_chunk": t.z_chunk}

    # -- probes and asynchronous read-back ---------------------------------------
    def set_probes(self, cells, capacity: int) -> None:
        """Ez and Hy at `cells` ((x, y, z) each) after every step, kept for the
        last `capacity` steps in device memory; no cells removes them."""
        flat = (C.c_uint32 * max(1, 3 * len(cells)))(*[int(v) for c in cells for v in c])
        _abi.check(_abi.lib().dp_sim_set_probes(self.handle, flat, len(cells), capacity))
        self.probe_count = len(cells)

    def read_probes(self, first_step: int, steps: int) -> np.ndarray:
        """steps × probes × (Ez, Hy) for steps first_step .. first_step+steps-1."""
        count = steps * self.probe_count * 2
        out = np.empty(max(count, 1), dtype=np.float32)
        _abi.check(_abi.lib().dp_sim_read_probes(self.handle, first_step, steps, out.ctypes.data, count))
        return out[:count].reshape(steps, self.probe_count, 2)

    def read_field_async(self, field: int, host_ptr: int, count: int) -> None:
        """Queues a read of `field` into host memory at `host_ptr` (pinned for
        overlap); the data is there after wait()."""
        _abi.check(_abi.lib().dp_sim_read_field_async(self.handle, field, C.c_void_p(host_ptr), count))

    def restore(self, snapshot: Snapshot) -> None:
        e = np.ascontiguousarray(snapshot.electric, dtype=np.float32)
        h = np.ascontiguousarray(snapshot.magnetic, dtype=np.float32)
        _abi.check(_abi.lib().dp_sim_restore(self.handle, snapshot.step, e.ctypes.data, h.ctypes.data, e.size))


class Simulation64:
    """The FP64 instance (dp_sim64): the same step in double on the GPU, the
    run the f32 step's error is measured against."""

    def __init__(self, scene: Scene | ResolvedScene, device: int = 0):
        self.resolved = scene if isinstance(scene, ResolvedScene) else ResolvedScene(scene)
        handle = C.c_void_p()
        _abi.check(_abi.lib().dp_sim64_create(self.resolved.handle, device, C.byref(handle)))
        self.handle = handle
        self.extent = self.resolved.extent
        self.cells = self.resolved.cells

    def __del__(self):
        if getattr(self, "handle", None):
            _abi.lib().dp_sim64_destroy(self.handle)
            self.handle = None

    def close(self) -> None:
        self.__del__()

    def advance_by(self, steps: int) -> None:
        _abi.check(_abi.lib().dp_sim64_advance(self.handle, steps))

    def wait(self, timeout_ms: int = 600_000) -> None:
        _abi.check(_abi.lib().dp_sim64_wait(self.handle, timeout_ms))

    def step_count(self) -> int:
        return _abi.lib().dp_sim64_step_count(self.handle)

    def _read(self, field: int) -> np.ndarray:
        out = np.empty(3 * self.cells, dtype=np.float64)
        _abi.check(_abi.lib().dp_sim64_read_field(self.handle, field, out.ctypes.data, out.size))
        return out

    def read_electric(self) -> np.ndarray:
        return self._read(_abi.DP_FIELD_ELECTRIC)

    def read_magnetic(self) -> np.ndarray:
        return self._read(_abi.DP_FIELD_MAGNETIC)

    def energy(self) -> Energy:
        e, m = C.c_double(), C.c_double()
        _abi.check(_abi.lib().dp_sim64_energy(self.handle, C.byref(e), C.byref(m)))
        return Energy(e.value, m.value)


def tuning_cache_export() -> str:
    """The process's tuned plans as text, one line per grid shape:
    "nx ny nz sms cells_per_lane tile_y ring_slots z_chunk ms_per_step"."""
    need = C.c_size_t()
    status = _abi.lib().dp_tune_cache_export(None, 0, C.byref(need))
    if status not in (_abi.DP_OK, _abi.DP_ERR_RANGE):
        _abi.check(status)
    buf = C.create_string_buffer(need.value + 1)
    _abi.check(_abi.lib().dp_tune_cache_export(buf, len(buf), C.byref(need)))
    return buf.value.decode()


def tuning_cache_import(text: str) -> None:
    """Adds exported lines to the process's tuned plans."""
    _abi.check(_abi.lib().dp_tune_cache_import(text.encode()))


def tuning_cache_clear() -> None:
    _abi.lib().dp_tune_cache_clear()
