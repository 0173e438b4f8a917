"""The batched form over the C ABI: many scenes advanced by one launch per step.

``Batch`` owns a device arena; ``add`` admits a resolved scene for a number of
steps (raising ``DiaphaneError`` DP_ERR_OOM when the arena cannot hold it
now), ``advance_chunk`` runs one K-step chunk for every scene with steps left,
and ``read_*`` return one scene's fields exactly as ``Simulation`` would.
"""
from __future__ import annotations

import ctypes as C
from typing import Sequence

import numpy as np

from . import _abi
from .simulation import ResolvedScene, _output


class Batch:
    def __init__(self, arena_bytes: int, chunk_steps: int = 50, max_scenes: int = 256, device: int = 0,
                 use_graphs: bool = True, cells_per_lane: int = 0, unit_planes: int = 0, check_finite: bool = True,
                 axis_order: int = 0):
        opts = _abi.dp_batch_options(device, chunk_steps, arena_bytes, max_scenes, int(use_graphs), cells_per_lane,
                                     unit_planes, int(not check_finite), axis_order)
        handle = C.c_void_p()
        _abi.check(_abi.lib().dp_batch_create(C.byref(opts), C.byref(handle)))
        self.handle = handle
        self.chunk_steps = chunk_steps
        self.scenes: dict[int, ResolvedScene] = {}
        self.probe_counts: dict[int, int] = {}

    def __del__(self):
        if getattr(self, "handle", None):
            _abi.lib().dp_batch_destroy(self.handle)
            self.handle = None

    def close(self) -> None:
        self.__del__()

    @staticmethod
    def bytes_for(resolved: ResolvedScene, steps: int, probe_count: int = 0) -> int:
        return _abi.lib().dp_scene_batch_bytes(resolved.handle, probe_count, steps)

    def add(self, resolved: ResolvedScene, steps: int, accumulate_intensity: bool = False,
            probes: Sequence[Sequence[int]] = ()) -> int:
        flat = (C.c_uint32 * max(1, 3 * len(probes)))(*[int(v) for p in probes for v in p])
        ident = C.c_uint64()
        _abi.check(_abi.lib().dp_batch_add(self.handle, resolved.handle, steps, int(accumulate_intensity), flat,
                                           len(probes), C.byref(ident)))
        self.scenes[ident.value] = resolved
        self.probe_counts[ident.value] = len(probes)
        return ident.value

    def remove(self, ident: int) -> None:
        _abi.check(_abi.lib().dp_batch_remove(self.handle, ident))
        self.scenes.pop(ident, None)
        self.probe_counts.pop(ident, None)

    def advance_chunk(self) -> int:
        stepping = C.c_uint32()
        _abi.check(_abi.lib().dp_batch_advance_chunk(self.handle, C.byref(stepping)))
        return stepping.value

    def run_to_completion(self) -> int:
        chunks = 0
        while self.advance_chunk():
            chunks += 1
        self.wait()
        return chunks

    def wait(self, timeout_ms: int = 600_000) -> None:
        _abi.check(_abi.lib().dp_batch_wait(self.handle, timeout_ms))

    def status(self, ident: int) -> tuple[int, int]:
        step, target = C.c_uint64(), C.c_uint64()
        _abi.check(_abi.lib().dp_batch_status(self.handle, ident, C.byref(step), C.byref(target)))
        return step.value, target.value

    def layout(self, ident: int) -> tuple[int, int]:
        """(axis order, tile width in cells) the batch stores a scene in;
        order 0 is the scene's own (xyz), 1-5 are yxz, xzy, zyx, yzx, zxy."""
        order, width = C.c_uint32(), C.c_uint32()
        _abi.check(_abi.lib().dp_batch_layout(self.handle, ident, C.byref(order), C.byref(width)))
        return order.value, width.value

    def fault(self, ident: int) -> tuple[int, int]:
        """(DP_OK, 0), or (DP_ERR_NONFINITE, the step count it stopped at)
        for a scene whose fields a per-chunk check found NaN or infinite:
        such a scene has stopped stepping; the others run on."""
        fault, at = C.c_int(), C.c_uint64()
        _abi.check(_abi.lib().dp_batch_fault(self.handle, ident, C.byref(fault), C.byref(at)))
        return fault.value, at.value

    def _read(self, ident: int, field: int, count: int, out=None) -> np.ndarray:
        out = _output(out, count)
        _abi.check(_abi.lib().dp_batch_read_field(self.handle, ident, field, out.ctypes.data, count))
        return out

    def read_electric(self, ident: int, out=None) -> np.ndarray:
        return self._read(ident, _abi.DP_FIELD_ELECTRIC, 3 * self.scenes[ident].cells, out)

    def read_magnetic(self, ident: int, out=None) -> np.ndarray:
        return self._read(ident, _abi.DP_FIELD_MAGNETIC, 3 * self.scenes[ident].cells, out)

    def read_intensity(self, ident: int, out=None) -> np.ndarray:
        return self._read(ident, _abi.DP_FIELD_INTENSITY, self.scenes[ident].cells, out)

    def read_probes(self, ident: int) -> np.ndarray:
        step, _ = self.status(ident)
        n = step * self.probe_counts[ident] * 2
        out = np.empty(n, dtype=np.float32)
        _abi.check(_abi.lib().dp_batch_read_probes(self.handle, ident, out.ctypes.data, n))
        return out.reshape(step, self.probe_counts[ident], 2)

    def memory(self) -> tuple[int, int]:
        used, cap = C.c_uint64(), C.c_uint64()
        _abi.check(_abi.lib().dp_batch_memory(self.handle, C.byref(used), C.byref(cap)))
        return used.value, cap.value

    def launch_count(self) -> int:
        return _abi.lib().dp_batch_launch_count(self.handle)
