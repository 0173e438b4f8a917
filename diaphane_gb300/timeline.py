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
