"""The served form: requests arrive over time, join a running batch at chunk
boundaries and leave when done.  Every request's probe series (Ez and Hy at
each probe cell after each step) must equal the oracle's run of that request
alone, whatever it shared the batch with."""
import numpy as np
import pytest

import oracle
from diaphane_gb300.serve import Server, poisson_trace, serve_plain, summary
from diaphane_gb300.workloads import mixed_scene

pytestmark = pytest.mark.gpu


def oracle_series(request, threads):
    scene = request.scene if request.scene is not None else mixed_scene(request.seed, request.lo, request.hi)
    ref = oracle.OracleSimulation(scene, threads=threads)
    out = np.empty((request.steps, len(request.probes), 2), dtype=np.float32)
    for t in range(request.steps):
        ref.advance()
        for k, p in enumerate(request.probes):
            out[t, k, 0] = ref.sample_electric(2, p)
            out[t, k, 1] = ref.sample_magnetic(1, p)
    return out


def test_requests_served_in_a_mix_match_each_run_alone(threads):
    trace = poisson_trace(6, rate=150.0, seed=0x7E57, lo=36, hi=60, steps=(40, 130), probe_count=4)
    server = Server(2 << 30, max_scenes=8, chunk_steps=16)
    server.serve(trace)
    assert server.peak_active >= 2  # the requests overlapped
    for r in trace:
        assert r.done is not None and r.done >= r.arrival
        assert r.series.shape == (r.steps, 4, 2)
        ref = oracle_series(r, threads)
        assert np.array_equal(r.series.view(np.uint32), ref.view(np.uint32)), r.ident
    used, _ = server.batch.memory()
    assert used == 0  # every request left and gave its bytes back
    server.close()


def test_admission_waits_for_bytes_to_free():
    """An arena that holds one request at a time serves them one after another."""
    trace = poisson_trace(3, rate=1000.0, seed=0xADD, lo=40, hi=48, steps=(30, 40), probe_count=2)
    for r in trace:
        r.resolve()
    from diaphane_gb300 import Batch
    biggest = max(Batch.bytes_for(r.resolved, r.steps, len(r.probes)) for r in trace)
    server = Server(biggest + (1 << 20), max_scenes=4, chunk_steps=8)
    server.serve(trace)
    assert server.peak_active == 1
    assert all(r.series is not None and r.series.shape[0] == r.steps for r in trace)
    server.close()


def test_plain_replay_and_summary():
    trace = serve_plain(poisson_trace(3, rate=1000.0, seed=0x9A1, lo=32, hi=40, steps=(20, 30)))
    s = summary(trace)
    assert s["requests"] == 3 and s["solves_per_s"] > 0 and s["p99_s"] >= s["p50_s"] > 0


def test_served_and_plain_replays_return_the_same_series():
    """The plain replay records the same probes through the solo solver's
    probe ring: every request's series is the same bits in both."""
    served = Server(1 << 30, max_scenes=8, chunk_steps=8)
    a = served.serve(poisson_trace(4, rate=1000.0, seed=0x5A3E, lo=32, hi=44, steps=(20, 36), probe_count=3))
    served.close()
    b = serve_plain(poisson_trace(4, rate=1000.0, seed=0x5A3E, lo=32, hi=44, steps=(20, 36), probe_count=3))
    for x, y in zip(sorted(a, key=lambda r: r.ident), sorted(b, key=lambda r: r.ident)):
        assert x.series.shape == y.series.shape == (x.steps, 3, 2)
        assert np.array_equal(x.series.view(np.uint32), y.series.view(np.uint32)), x.ident


def gain_scene(seed):
    """A mixed scene with a block of gain medium (conductivity -9 S/m: an
    electric loss of about -0.97, so E there grows ~60x a step) at its
    centre.  On the oracle its fields are non-finite by step 48."""
    from diaphane_gb300 import Material, Shape
    scene = mixed_scene(seed, 36, 48)
    gain = scene.materials.push(Material(relative_permittivity=1.0, conductivity=-9.0))
    scene.shapes.append(Shape.block((0.0, 0.0, 0.0), (0.016, 0.016, 0.016), gain))
    return scene


def test_a_non_finite_scene_stops_and_the_one_beside_it_runs_on(threads):
    """The batch's per-chunk check (is_finite, src/cpu.rs:707-713): the gain
    scene stops with DP_ERR_NONFINITE within two chunks of going non-finite,
    and a healthy scene in the same batch runs to its end, bit-identical to
    the oracle's run of it alone."""
    from diaphane_gb300 import Batch, ResolvedScene
    from diaphane_gb300._abi import DP_ERR_NONFINITE
    batch = Batch(1 << 30, chunk_steps=16, max_scenes=4)
    bad = batch.add(ResolvedScene(gain_scene(7)), 400)
    good_scene = mixed_scene(8, 36, 48)
    good = batch.add(ResolvedScene(good_scene), 400)
    batch.run_to_completion()
    fault, at = batch.fault(bad)
    assert fault == DP_ERR_NONFINITE and 0 < at <= 48 + 3 * 16, (fault, at)
    assert batch.status(bad) == (at, at)
    assert batch.fault(good) == (0, 0) and batch.status(good) == (400, 400)
    ref = oracle.OracleSimulation(good_scene, threads=threads)
    ref.advance_by(400)
    assert np.array_equal(batch.read_electric(good).view(np.uint32), ref.read_electric().view(np.uint32))
    batch.close()


def test_a_failing_request_and_a_cancelled_one_leave_the_others_exact(threads):
    """One request's fields turn non-finite (the gain block) and another's
    client gives up mid-run: the first is retired as failed, the second is
    removed from the batch, and every other request's probe series is still
    bit-identical to the oracle's run of it alone."""
    trace = poisson_trace(6, rate=400.0, seed=0xFA17, lo=36, hi=52, steps=(120, 200), probe_count=3)
    trace[1].scene = gain_scene(trace[1].seed)
    trace[1].steps = 600
    trace[3].steps = 20_000
    trace[3].cancel_after = 0.05
    server = Server(2 << 30, max_scenes=8, chunk_steps=16)
    server.serve(trace)
    assert trace[1].outcome == "failed" and 0 < trace[1].fault_step < trace[1].steps
    assert trace[3].outcome == "cancelled" and trace[3].series is None
    for r in trace:
        if r.ident in (1, 3):
            continue
        assert r.outcome == "done"
        ref = oracle_series(r, threads)
        assert np.array_equal(r.series.view(np.uint32), ref.view(np.uint32)), r.ident
    s = summary(trace)
    assert s["solved"] == 4 and s["failed"] == 1 and s["cancelled"] == 1
    used, _ = server.batch.memory()
    assert used == 0
    server.close()
