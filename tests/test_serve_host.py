"""The served loop's host logic without a GPU: `Server.serve` driven against a
fake batch and a fake clock.  Admission in arrival order while bytes and
slots allow, waiting (not failing) on DP_ERR_OOM / DP_ERR_BUSY while another
request can still leave, failing when nothing can, and each request leaving
with its series at the chunk where its last step ran, a scene that the
batch's finiteness check stopped retired as failed, and a request whose
client gave up dropped from the queue or the batch as cancelled."""
from types import SimpleNamespace

import numpy as np
import pytest

import diaphane_gb300.serve as serve_mod
from diaphane_gb300._abi import DP_ERR_BUSY, DP_ERR_NONFINITE, DP_ERR_OOM, DiaphaneError
from diaphane_gb300.serve import Request, Server, summary


class FakeClock:
    def __init__(self, tick=0.001):
        self.now = 0.0
        self.tick = tick

    def __call__(self):
        self.now += self.tick
        return self.now

    def sleep(self, seconds):
        self.now += max(0.0, seconds)


class FakeBatch:
    """Admission by bytes and slots, `chunk` steps per advance, a series of
    the scene's id at every step; a scene named in `blow_up` (name -> step)
    is stopped by the finiteness check at the first chunk past that step."""

    def __init__(self, slots, capacity, chunk=10, blow_up=None):
        self.slots, self.capacity, self.chunk = slots, capacity, chunk
        self.blow_up = blow_up or {}
        self.faults = {}
        self.active = {}
        self.used = 0
        self.next_id = 0
        self.log = []

    def add(self, resolved, steps, probes=()):
        if len(self.active) >= self.slots:
            raise DiaphaneError(DP_ERR_BUSY, "every scene slot is in use")
        if self.used + resolved.bytes > self.capacity:
            raise DiaphaneError(DP_ERR_OOM, "the arena cannot hold this scene now")
        ident = self.next_id
        self.next_id += 1
        self.active[ident] = [0, steps, resolved.bytes, resolved.name]
        self.used += resolved.bytes
        self.log.append(("add", resolved.name))
        return ident

    def status(self, ident):
        step, target = self.active[ident][:2]
        return step, target

    def fault(self, ident):
        return self.faults.get(ident, (0, 0))

    def advance_chunk(self):
        for ident, entry in self.active.items():
            entry[0] = min(entry[1], entry[0] + self.chunk)
            at = self.blow_up.get(entry[3])
            if at is not None and entry[0] >= at and ident not in self.faults:
                self.faults[ident] = (DP_ERR_NONFINITE, entry[0])
                entry[1] = entry[0]  # stops stepping: looks finished
        return len(self.active)

    def wait(self, timeout_ms=0):
        pass

    def read_probes(self, ident):
        return np.full((self.active[ident][1], 1, 2), float(ident), np.float32)

    def remove(self, ident):
        self.used -= self.active.pop(ident)[2]
        self.log.append(("remove", ident))

    def close(self):
        pass


def make_server(batch, clock, monkeypatch):
    monkeypatch.setattr(serve_mod, "time", SimpleNamespace(sleep=clock.sleep, perf_counter=clock))
    server = Server.__new__(Server)
    server.batch = batch
    server.clock = clock
    server.chunks = 0
    server.busy_seconds = 0.0
    server.peak_active = 0
    return server


def requests(specs):
    """(arrival, steps, bytes) per request, already resolved."""
    out = []
    for k, (arrival, steps, nbytes) in enumerate(specs):
        r = Request(k, arrival, seed=k, steps=steps, probe_count=1)
        r.resolved = SimpleNamespace(bytes=nbytes, name=k)
        r.cells = 1000
        r.probes = [(0, 0, 0)]
        out.append(r)
    return out


def test_requests_join_in_arrival_order_and_leave_with_their_series(monkeypatch):
    clock = FakeClock()
    batch = FakeBatch(slots=8, capacity=1 << 30, chunk=10)
    server = make_server(batch, clock, monkeypatch)
    trace = requests([(0.0, 350, 10), (0.005, 120, 10), (0.002, 500, 10), (0.3, 80, 10)])
    server.serve(trace)
    adds = [name for kind, name in batch.log if kind == "add"]
    assert adds == [0, 2, 1, 3]  # arrival order
    for r in trace:
        assert r.series is not None and r.series.shape == (r.steps, 1, 2)
        assert r.arrival <= r.admitted <= r.done
        assert r.latency > 0
    assert not batch.active and batch.used == 0
    assert server.peak_active >= 2
    s = summary(trace)
    assert s["requests"] == 4 and s["p99_s"] >= s["p50_s"] > 0


def test_admission_waits_for_bytes_to_free(monkeypatch):
    clock = FakeClock()
    batch = FakeBatch(slots=8, capacity=100, chunk=10)
    server = make_server(batch, clock, monkeypatch)
    trace = requests([(0.0, 20, 60), (0.0, 20, 60), (0.0, 20, 60)])
    server.serve(trace)
    assert server.peak_active == 1
    kinds = [kind for kind, _ in batch.log]
    assert kinds == ["add", "remove", "add", "remove", "add", "remove"]
    assert all(r.series is not None for r in trace)


def test_admission_waits_for_a_free_slot(monkeypatch):
    clock = FakeClock()
    batch = FakeBatch(slots=2, capacity=1 << 30, chunk=5)
    server = make_server(batch, clock, monkeypatch)
    trace = requests([(0.0, 10 + 5 * k, 1) for k in range(6)])
    server.serve(trace)
    assert server.peak_active == 2
    assert all(r.series is not None for r in trace)


def test_a_request_no_arena_can_hold_fails_when_nothing_can_leave(monkeypatch):
    clock = FakeClock()
    batch = FakeBatch(slots=8, capacity=100, chunk=10)
    server = make_server(batch, clock, monkeypatch)
    with pytest.raises(DiaphaneError) as err:
        server.serve(requests([(0.0, 20, 500)]))
    assert err.value.status == DP_ERR_OOM


def test_idle_time_waits_for_the_next_arrival(monkeypatch):
    clock = FakeClock()
    batch = FakeBatch(slots=8, capacity=1 << 30, chunk=10)
    server = make_server(batch, clock, monkeypatch)
    trace = requests([(0.0, 10, 1), (5.0, 10, 1)])
    server.serve(trace)
    late = trace[1]
    assert late.admitted >= 5.0 and late.done >= late.admitted


def test_a_failing_request_is_retired_as_failed_and_the_others_finish(monkeypatch):
    clock = FakeClock()
    batch = FakeBatch(slots=8, capacity=1 << 30, chunk=10, blow_up={1: 35})
    server = make_server(batch, clock, monkeypatch)
    trace = requests([(0.0, 200, 10), (0.0, 200, 10), (0.0, 120, 10)])
    server.serve(trace)
    assert trace[1].outcome == "failed" and trace[1].fault_step == 40 and trace[1].series is None
    for r in (trace[0], trace[2]):
        assert r.outcome == "done" and r.series.shape == (r.steps, 1, 2)
    assert not batch.active and batch.used == 0
    s = summary(trace)
    assert s["solved"] == 2 and s["failed"] == 1 and s["cancelled"] == 0


def test_a_client_that_gives_up_is_dropped_from_the_queue_or_the_batch(monkeypatch):
    clock = FakeClock(tick=0.01)
    batch = FakeBatch(slots=1, capacity=1 << 30, chunk=10)
    server = make_server(batch, clock, monkeypatch)
    # 0 runs long and gives up mid-run; 1 waits behind it for the one slot and
    # gives up while queued; 2 is solved once 0 has left.
    trace = requests([(0.0, 10_000, 1), (0.0, 10, 1), (0.0, 30, 1)])
    trace[0].cancel_after = 0.5
    trace[1].cancel_after = 0.2
    server.serve(trace)
    assert [r.outcome for r in trace] == ["cancelled", "cancelled", "done"]
    assert trace[0].series is None and trace[1].series is None and trace[1].admitted is None
    assert ("remove", 0) in batch.log and trace[0].done >= 0.5
    assert not batch.active and batch.used == 0
    assert summary(trace)["cancelled"] == 2
