"""Keyframe timeline over any Steppable solver (src/timeline.rs:74-213).

A caller of the step path, not part of it: seeking backwards restores the
newest keyframe at or before the target and replays, or resets and replays
from the start when the window has slid past it.
"""
from __future__ import annotations

from collections import deque
from dataclasses import dataclass


@dataclass(frozen=True)
class Seek:
    """src/timeline.rs:83-106: what a seek had to do."""
    kind: str  # "unchanged" | "forward" | "keyframe" | "start"
    replayed: int = 0
    at: int | None = None


class Timeline:
    def __init__(self, interval: int, capacity: int):
        if interval <= 0:
            raise ValueError("keyframe interval must be positive")
        if capacity <= 0:
            raise ValueError("a timeline needs room for at least one keyframe")
        self.keyframes: deque = deque()
        self.interval = interval
        self.capacity = capacity

    def observe(self, simulation) -> None:
        """src/timeline.rs:137-154: records when the step crosses an interval."""
        step = simulation.step_count()
        if self.keyframes:
            last = self.keyframes[-1].step
            if step <= last:
                return
            newest = last // self.interval
        else:
            newest = 0
        if step // self.interval <= newest:
            return
        if len(self.keyframes) == self.capacity:
            self.keyframes.popleft()
        self.keyframes.append(simulation.snapshot())

    def clear(self) -> None:
        self.keyframes.clear()

    def earliest(self) -> int | None:
        return self.keyframes[0].step if self.keyframes else None

    def keyframe_count(self) -> int:
        return len(self.keyframes)

    def bytes(self) -> int:
        return sum(k.bytes() for k in self.keyframes)

    def seek(self, simulation, target: int) -> Seek:
        """src/timeline.rs:180-212."""
        current = simulation.step_count()
        if target == current:
            return Seek("unchanged")
        if target > current:
            simulation.advance_by(target - current)
            return Seek("forward", target - current)
        for frame in reversed(self.keyframes):
            if frame.step <= target:
                simulation.restore(frame)
                simulation.advance_by(target - frame.step)
                return Seek("keyframe", target - frame.step, frame.step)
        simulation.reset()
        simulation.advance_by(target)
        return Seek("start", target)


_SEEK_KINDS = {0: "unchanged", 1: "forward", 2: "keyframe", 3: "start"}


class DeviceTimeline:
    """The same keyframe ring with its keyframes in device memory
    (dp_keyframes): snapshot and restore are device-to-device copies on the
    simulation's stream.  Bound to one Simulation, which must outlive it."""

    def __init__(self, simulation, interval: int, capacity: int):
        from . import _abi
        import ctypes as C
        self._abi, self._C = _abi, C
        self.simulation = simulation
        handle = C.c_void_p()
        _abi.check(_abi.lib().dp_keyframes_create(simulation.handle, interval, capacity, C.byref(handle)))
        self.handle = handle
        self.interval = interval
        self.capacity = capacity

    def __del__(self):
        if getattr(self, "handle", None):
            self._abi.lib().dp_keyframes_destroy(self.handle)
            self.handle = None

    def close(self) -> None:
        self.__del__()

    def _bound(self, simulation) -> None:
        if simulation is not None and simulation is not self.simulation:
            raise ValueError("a device timeline serves the simulation it was created for")

    def observe(self, simulation=None) -> None:
        self._bound(simulation)
        self._abi.check(self._abi.lib().dp_keyframes_observe(self.handle))

    def seek(self, simulation, target: int) -> Seek:
        self._bound(simulation)
        out = self._abi.dp_seek()
        self._abi.check(self._abi.lib().dp_keyframes_seek(self.handle, target, self._C.byref(out)))
        kind = _SEEK_KINDS[out.kind]
        return Seek(kind, out.replayed, out.at if kind == "keyframe" else None)

    def clear(self) -> None:
        self._abi.check(self._abi.lib().dp_keyframes_clear(self.handle))

    def earliest(self) -> int | None:
        if self.keyframe_count() == 0:
            return None
        step = self._C.c_uint64()
        self._abi.check(self._abi.lib().dp_keyframes_earliest(self.handle, self._C.byref(step)))
        return step.value

    def keyframe_count(self) -> int:
        return self._abi.lib().dp_keyframes_count(self.handle)

    def bytes(self) -> int:
        return self._abi.lib().dp_keyframes_bytes(self.handle)
