"""Headless volume rendering of a live simulation (dp_renderer).

The reference viewer's volume pass and exposure control, drawing into an
RGBA8 image in device memory; ``pixels()`` reads it back and ``write_png``
stores it.  The renderer borrows the simulation's field buffers, so a frame
costs no copies of the fields.
"""
from __future__ import annotations

import ctypes as C
import struct
import zlib
from dataclasses import dataclass

import numpy as np

from . import _abi

MODES = {"energy": _abi.DP_VIEW_ENERGY, "electric": _abi.DP_VIEW_ELECTRIC, "magnetic": _abi.DP_VIEW_MAGNETIC,
         "magnitude": _abi.DP_VIEW_MAGNITUDE, "fields": _abi.DP_VIEW_FIELDS, "grid": _abi.DP_VIEW_GRID,
         "ribbons": _abi.DP_VIEW_RIBBONS, "intensity": _abi.DP_VIEW_INTENSITY}


@dataclass
class View:
    """Camera::new and ViewSettings::new (examples/common/camera.rs, render.rs)."""
    yaw: float = 0.9
    pitch: float = 0.45
    distance: float = 1.9
    fov: float = 0.8
    mode: int = _abi.DP_VIEW_FIELDS
    gain: float = 1.0
    log_strength: float = 6.0
    scrub: bool = False
    played: float = 0.0
    window_start: float = 0.0

    def c(self) -> _abi.dp_view:
        return _abi.dp_view(self.yaw, self.pitch, self.distance, self.fov, self.mode, self.gain, self.log_strength,
                            int(self.scrub), self.played, self.window_start)


class Renderer:
    def __init__(self, simulation, width: int, height: int):
        handle = C.c_void_p()
        _abi.check(_abi.lib().dp_renderer_create(simulation.handle, width, height, C.byref(handle)))
        self.handle = handle
        self.simulation = simulation
        self.width, self.height = width, height

    def __del__(self):
        if getattr(self, "handle", None):
            _abi.lib().dp_renderer_destroy(self.handle)
            self.handle = None

    def close(self) -> None:
        self.__del__()

    def measure(self) -> None:
        _abi.check(_abi.lib().dp_renderer_measure(self.handle))

    def draw(self, view: View | None = None, advanced: bool = True) -> None:
        v = (view or View()).c()
        _abi.check(_abi.lib().dp_renderer_draw(self.handle, C.byref(v), int(advanced)))

    def pixels(self) -> np.ndarray:
        out = np.empty((self.height, self.width, 4), np.uint8)
        _abi.check(_abi.lib().dp_renderer_pixels(self.handle, out.ctypes.data, out.nbytes))
        return out

    def image_ptr(self) -> int:
        p = C.c_void_p()
        _abi.check(_abi.lib().dp_renderer_image(self.handle, C.byref(p)))
        return p.value

    def state(self) -> tuple[np.ndarray, float, tuple[int, int]]:
        peaks = (C.c_float * 8)()
        scale = C.c_float()
        comps = (C.c_uint32 * 2)()
        _abi.check(_abi.lib().dp_renderer_state(self.handle, peaks, C.byref(scale), comps))
        return np.array(peaks, np.float32), scale.value, (comps[0], comps[1])


def write_png(path, rgba: np.ndarray) -> None:
    """An RGBA8 image as a PNG (sRGB), with no dependency beyond zlib."""
    h, w, _ = rgba.shape
    raw = b"".join(b"\x00" + rgba[y].tobytes() for y in range(h))

    def chunk(kind: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n")
        f.write(chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 6, 0, 0, 0)))
        f.write(chunk(b"sRGB", b"\x00"))
        f.write(chunk(b"IDAT", zlib.compress(raw, 6)))
        f.write(chunk(b"IEND", b""))
