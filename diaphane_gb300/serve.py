"""The served form: solve requests arrive over time and join a running batch.

A request names a scene (built from its seed), a step count and probe cells.
``Server.serve`` replays an arrival trace against one ``Batch``: requests that
have arrived are admitted in arrival order while the arena's bytes and the
batch's scene slots hold them; the batch advances one chunk at a time; a
request leaves at the chunk boundary where its last step ran, and its probe
series (Ez and Hy at every probe cell after every step) is read back.  A
scene joins and leaves only between chunks, so its result is the same alone
or in any mix.

Failures stay with their request: a scene whose fields turn NaN or infinite
is stopped by the batch's per-chunk check (is_finite, src/cpu.rs:707-713) and
retired as "failed" with the step it stopped at, and a request whose client
gives up (``cancel_after`` seconds after arrival) leaves the queue, or the
batch at the next chunk boundary, as "cancelled"; the other requests run on.

``serve_plain`` replays the same trace against the one-scene-at-a-time solver
(``Simulation``): first come, first served, each request stepped to the end
before the next one starts.
"""
from __future__ import annotations

import math
import time
from collections import deque
from dataclasses import dataclass, field
from typing import Callable, Optional

import numpy as np

from ._abi import DiaphaneError, DP_ERR_BUSY, DP_ERR_OOM, DP_OK
from .batch import Batch
from .scene import Scene
from .simulation import ResolvedScene, Simulation
from .workloads import SplitMix64, mixed_scene


@dataclass
class Request:
    ident: int
    arrival: float              # seconds after the trace starts
    seed: int                   # scene seed
    steps: int
    probe_count: int = 8
    lo: int = 48                # axis range of the scene, cells
    hi: int = 320
    scene: Optional[Scene] = None          # an explicit scene instead of the seed's
    cancel_after: Optional[float] = None   # the client gives up this many seconds after arrival
    # Filled in by a replay.
    resolved: Optional[ResolvedScene] = None
    probes: list = field(default_factory=list)
    cells: int = 0
    admitted: Optional[float] = None
    done: Optional[float] = None
    series: Optional[np.ndarray] = None   # steps × probes × (Ez, Hy); None unless "done"
    outcome: str = ""                     # "done", "failed" (non-finite fields) or "cancelled"
    fault_step: Optional[int] = None      # steps run when a failed request was stopped

    def resolve(self) -> ResolvedScene:
        if self.resolved is None:
            scene = self.scene if self.scene is not None else mixed_scene(self.seed, self.lo, self.hi)
            self.resolved = ResolvedScene(scene)
            n = self.resolved.extent
            self.cells = self.resolved.cells
            rng = SplitMix64(self.seed ^ 0x9B0B_E5)
            self.probes = [tuple(int(rng.uniform(0, n[a])) % n[a] for a in range(3)) for _ in range(self.probe_count)]
        return self.resolved

    @property
    def latency(self) -> float:
        return self.done - self.arrival

    def gave_up(self, now: float) -> bool:
        return self.cancel_after is not None and now >= self.arrival + self.cancel_after


def poisson_trace(count: int, rate: float, seed: int = 0x5E_4E_D0, lo: int = 48, hi: int = 320,
                  steps: tuple[int, int] = (200, 5000), probe_count: int = 8) -> list[Request]:
    """`count` requests with exponential inter-arrival gaps of mean 1/rate s,
    scene axes log-uniform in [lo, hi] and step counts uniform in `steps`."""
    rng = SplitMix64(seed)
    t = 0.0
    out = []
    for k in range(count):
        t += -math.log(1.0 - rng.uniform(0.0, 1.0)) / rate
        n = int(rng.uniform(steps[0], steps[1] + 1))
        out.append(Request(k, t, (seed << 16) + k, min(n, steps[1]), probe_count, lo, hi))
    return out


class Server:
    """Continuous batching over one ``Batch``."""

    def __init__(self, arena_bytes: int, max_scenes: int = 256, chunk_steps: int = 50, device: int = 0,
                 clock: Callable[[], float] = time.perf_counter):
        self.batch = Batch(arena_bytes, chunk_steps=chunk_steps, max_scenes=max_scenes, device=device)
        self.clock = clock
        self.chunks = 0
        self.busy_seconds = 0.0
        self.peak_active = 0

    def close(self) -> None:
        self.batch.close()

    def _admit(self, queue: deque, active: dict, now: float) -> None:
        while queue:
            r = queue[0]
            try:
                ident = self.batch.add(r.resolve(), r.steps, probes=r.probes)
            except DiaphaneError as err:
                if err.status in (DP_ERR_OOM, DP_ERR_BUSY) and active:
                    return  # waits for a request to leave
                raise
            r.admitted = now
            active[ident] = r
            queue.popleft()

    def _finished(self, active: dict) -> list:
        done = []
        for ident in active:
            issued, target = self.batch.status(ident)
            if issued >= target:
                done.append(ident)
        return done

    def _retire(self, active: dict, finished: list, t0: float) -> None:
        for ident in finished:
            r = active.pop(ident)
            fault, at = self.batch.fault(ident)
            if fault == DP_OK:
                r.series = self.batch.read_probes(ident)  # waits for the chunk that finished it
                r.outcome = "done"
            else:
                r.outcome, r.fault_step = "failed", at
            self.batch.remove(ident)
            r.done = self.clock() - t0
            r.resolved = None  # the host copy of the scene is no longer needed

    def _cancel(self, queue: deque, active: dict, now: float) -> None:
        """Requests whose client has given up leave the queue, or the batch
        (after the chunk that is running), without a result."""
        for r in [q for q in queue if q.gave_up(now)]:
            queue.remove(r)
            r.outcome, r.done, r.resolved = "cancelled", now, None
        for ident in [i for i, r in active.items() if r.gave_up(now)]:
            r = active.pop(ident)
            self.batch.remove(ident)
            r.outcome, r.done, r.resolved = "cancelled", now, None

    def serve(self, trace: list[Request]) -> list[Request]:
        pending = deque(sorted(trace, key=lambda r: r.arrival))
        queue: deque = deque()
        active: dict = {}
        t0 = self.clock()
        while pending or queue or active:
            now = self.clock() - t0
            while pending and pending[0].arrival <= now:
                queue.append(pending.popleft())
            self._cancel(queue, active, now)
            self._admit(queue, active, now)
            self.peak_active = max(self.peak_active, len(active))
            if active:
                c0 = self.clock()
                self.batch.advance_chunk()  # queued; at most two chunks run ahead of the host
                self.chunks += 1
                # Host scene setup of the next arrivals overlaps the chunk.
                for r in list(pending)[:4]:
                    if r.arrival <= self.clock() - t0 + 0.05:
                        r.resolve()
                # Wait only when a request's last step was just issued (or a
                # failed one was stopped).
                finished = self._finished(active)
                if finished:
                    self.batch.wait()
                    self._retire(active, finished, t0)
                self.busy_seconds += self.clock() - c0
            elif pending:
                pending[0].resolve()
                delay = pending[0].arrival - (self.clock() - t0)
                if delay > 0:
                    time.sleep(delay)
        return trace


def serve_plain(trace: list[Request], device: int = 0, clock: Callable[[], float] = time.perf_counter
                ) -> list[Request]:
    """First come, first served with one ``Simulation`` per request, each
    recording the same probe series as the served form (a probe ring of the
    request's step count) and reading it back when its last step has run.
    A request whose client gave up before its turn is skipped; one whose
    fields end non-finite is "failed"."""
    t0 = clock()
    for r in sorted(trace, key=lambda q: q.arrival):
        now = clock() - t0
        if now < r.arrival:
            time.sleep(r.arrival - now)
            now = clock() - t0
        if r.gave_up(now):
            r.outcome, r.done, r.resolved = "cancelled", now, None
            continue
        r.admitted = now
        sim = Simulation(r.resolve(), device=device)
        sim.set_probes(r.probes, capacity=r.steps)
        sim.advance_by(r.steps)
        if sim.is_finite():
            r.series = sim.read_probes(1, r.steps)
            r.outcome = "done"
        else:
            r.outcome, r.fault_step = "failed", r.steps
        sim.close()
        r.done = clock() - t0
        r.resolved = None
    return trace


def summary(trace: list[Request]) -> dict:
    """Solves per second and completion latency over the requests that
    were solved; failed and cancelled ones are counted beside them."""
    solved = [r for r in trace if r.outcome in ("done", "")]
    lat = np.array([r.latency for r in solved]) if solved else np.zeros(1)
    first = min(r.arrival for r in trace)
    last = max(r.done for r in trace)
    cell_steps = sum(r.steps * r.cells for r in solved)
    return {"requests": len(trace), "solved": len(solved),
            "failed": sum(r.outcome == "failed" for r in trace),
            "cancelled": sum(r.outcome == "cancelled" for r in trace),
            "solves_per_s": len(solved) / (last - first),
            "p50_s": float(np.percentile(lat, 50)), "p99_s": float(np.percentile(lat, 99)),
            "mean_s": float(lat.mean()), "makespan_s": last - first,
            "gcells_per_s": cell_steps / (last - first) / 1e9}
