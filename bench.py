"""Benchmark: Gcell-updates/s of the fused Yee step on the heterogeneous 512³ scene.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Workload (both arms): uniform 512³ grid at 1 mm, FP32, 10-cell absorbing
layer, 200 seeded dielectric spheres (radius 4-24 cells, εr in [1, 4]), a
perfectly conducting sphere of radius 40 cells, a matched lossy slab, and an
x-travelling total-field/scattered-field plane wave 16 cells inside the
absorber (Gaussian pulse, 10 cells per wavelength), intensity accumulation on.
A step is one full time step (H, sources, E, sources, intensity) of the whole
grid.  Synthetic data: the scene is generated from a fixed SplitMix64 seed.

ours:       the CUDA library through its C ABI.  `value` is device-timed
            (CUDA events on the simulation's stream) with the fields resident
            in HBM; the fields (6.4 GB) dwarf L2, so no flush is needed.
            `e2e` times the public API end to end with host buffers: restore
            the fields (the run's input state) from pinned host memory,
            advance K steps accumulating intensity, read the intensity (the
            run's result) back.
reference:  the reference's CPU path (its Rust toolchain is absent, so the
            oracle's C++ restatement of src/cpu.rs), on every host core, on
            the same scene, for as many steps as fit a bounded time budget.

N > 1 runs independent replicas (the step has no exchange to shard), one
process per GPU under torchrun; `value` sums all ranks' cells over the
slowest rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import platform
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

BYTES_PER_CELL = 48  # 6 f32 components read once and written once (benches/throughput.rs:17-18)
WORKLOAD = "heterogeneous scatterers 512^3"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2000)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", choices=["ours", "reference"], default="ours")
    p.add_argument("--side", type=int, default=512, help="grid side (512 is the workload; smaller for checks)")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--variant", default="",
                   help="fused kernel cx,tile_y,slots[,z_chunk] (default: tuned)")
    p.add_argument("--no-cpu", action="store_true")
    p.add_argument("--no-batched", action="store_true", help="skip the mixed-size batch measurement")
    p.add_argument("--no-served", action="store_true", help="skip the served-stream measurement")
    p.add_argument("--no-accuracy", action="store_true", help="skip the FP64 error measurement")
    p.add_argument("--no-tune", action="store_true", help="keep the planner's plan (no autotuning before timing)")
    p.add_argument("--regime", type=int, default=1000,
                   help="untimed steps before the warm-up, so the timed window sees the late-regime field "
                        "(the wave has filled the box and the absorbers hold decaying field)")
    p.add_argument("--workload", choices=["heterogeneous", "batched", "served", "accuracy", "extras", "kernels"],
                   default="heterogeneous")
    p.add_argument("--scenes", type=int, default=256, help="batched: scenes per batch")
    p.add_argument("--batch-steps", type=int, default=1000, help="batched: steps per scene")
    p.add_argument("--rates", default="4,16,64", help="served: arrival rates to sweep, requests/s")
    p.add_argument("--requests", type=int, default=48, help="served: requests per trace")
    p.add_argument("--ref-budget", type=float, default=60.0, help="reference arm: seconds of CPU stepping")
    return p.parse_args()


def measured_peaks() -> tuple[float, str]:
    path = ROOT / "MEASURED_PEAKS.json"
    if path.exists():
        try:
            return float(json.loads(path.read_text())["hbm_gbs"]), "measured"
        except Exception:
            pass
    return 6800.0, "fallback"


def profiled_traffic(side: int) -> float | None:
    """DRAM bytes per launch from the committed ncu summary, when one exists."""
    path = ROOT / "profiles" / "fused_step_heterogeneous.md"
    if not path.exists():
        return None
    for line in path.read_text().splitlines():
        if line.startswith("dram_bytes_per_launch_512:") and side == 512:
            return float(line.split(":", 1)[1].strip())
    return None


def config(side: int, n: int) -> dict:
    return {"workload": WORKLOAD if side == 512 else f"heterogeneous scatterers {side}^3",
            "grid": [side, side, side], "spheres": 200, "materials": 203, "intensity": True,
            "source": "TFSF box 16 cells inside the absorber (faces at cells 26 and 485), x-travelling plane wave",
            "boundary": "absorbing, 10 cells",
            "l2": f"inputs larger than L2 (fields {48 * side ** 3 / 1e9:.2f} GB per step), no flush",
            "parallelism": f"replicas{n}"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                                          "-lms", "200", "-i", str(self.index)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.reader = threading.Thread(target=self._read, daemon=True)
            self.reader.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.reader.join(timeout=2)

    def summary(self) -> dict:
        mhz, maxes, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                mhz.append(float(parts[1]))
                maxes.append(float(parts[2]))
            except ValueError:
                continue
            for name, flag in zip(names, parts[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(mhz) if mhz else None, "sm_max_mhz": max(maxes) if maxes else None,
                "reasons": sorted(reasons), "samples": len(mhz)}


def distributed():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def max_over_ranks(value: float, world: int) -> float:
    """The largest of every rank's value (the slowest rank's time): one
    all-reduce on the process group's own backend."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    device = f"cuda:{torch.cuda.current_device()}" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def partition(count: int, rank: int, world: int) -> list:
    """The units (scenes, requests) rank `rank` of `world` replicas runs:
    round robin, disjoint, covering all of them; no data crosses ranks."""
    return list(range(rank, count, max(world, 1)))


def cpu_port_rate(scene, threads: int, budget_s: float, max_steps: int, warmup: int) -> tuple[float, int, float]:
    """Oracle steps on `threads` host cores until the budget is spent."""
    import oracle
    sim = oracle.OracleSimulation(scene, threads=threads)
    sim.set_accumulate_intensity(True)
    if warmup:
        sim.advance_by(warmup)
    steps, start = 0, time.perf_counter()
    while steps < max_steps:
        sim.advance_by(1)
        steps += 1
        if time.perf_counter() - start > budget_s:
            break
    elapsed = time.perf_counter() - start
    cells = sim.cells
    return cells * steps / elapsed / 1e9, steps, elapsed


def cpu_model() -> str:
    """The host CPU's model name (lscpu, else /proc/cpuinfo)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    try:
        for line in Path("/proc/cpuinfo").read_text().splitlines():
            if line.lower().startswith(("model name", "cpu model")):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.processor() or platform.machine()


def loaded_libraries() -> list[str]:
    """The in-tree shared libraries this process has mapped (from
    /proc/self/maps), relative to the repository root."""
    found = set()
    try:
        for line in Path("/proc/self/maps").read_text().splitlines():
            path = line.split()[-1] if line.split() else ""
            if path.endswith(".so") and path.startswith(str(ROOT)):
                found.add(str(Path(path).relative_to(ROOT)))
    except OSError:
        pass
    return sorted(found)


def run_reference(args):
    world, rank, _ = distributed()
    if rank != 0:
        return
    # The scene is built with the oracle's grid resolver, so this process
    # never loads the CUDA library: the arm is the CPU restatement alone.
    import oracle
    from diaphane_gb300 import scene as scene_model, workloads
    scene_model.use_grid_resolver(oracle.OracleGridResolver)
    threads = os.cpu_count() or 1
    scene = workloads.heterogeneous(args.side)
    rate, steps, elapsed = cpu_port_rate(scene, threads, budget_s=args.ref_budget, max_steps=args.steps,
                                         warmup=args.warmup)
    sample = (f"{steps} oracle steps of the full {args.side}^3 scene in {elapsed:.1f} s "
              f"(time-budgeted; the per-step cost is constant)")
    line = {"impl": "reference", "metric": "Gcell-updates/s", "value": rate, "unit": "Gcell/s", "n_gpus": world,
            "steps": steps, "warmup": args.warmup, "ms_per_step": 1e3 * elapsed / max(steps, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded SplitMix64 scene)", "config": config(args.side, world),
            "cpu_baseline": {"value": rate, "unit": "Gcell/s", "cores": threads, "kind": "port", "sample": sample,
                             "nproc": os.cpu_count(), "cpu_model": cpu_model()},
            "e2e": {"value": rate, "unit": "Gcell/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "note": "reference is Rust (cargo absent on both machines); this is the oracle's C++ restatement "
                    "of src/cpu.rs with OpenMP over z planes",
            "libraries_loaded": loaded_libraries()}
    print(json.dumps(line), flush=True)


def run_ours(args):
    import numpy as np
    import torch

    world, rank, local = distributed()
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", init_method="env://")
    device = local if world > 1 else 0

    from diaphane_gb300 import DP_KERNEL_AUTO, ResolvedScene, Simulation, workloads
    from diaphane_gb300.build import build
    build()

    scene = workloads.heterogeneous(args.side)
    resolved = ResolvedScene(scene)
    v = ([int(t) for t in args.variant.split(",")] if args.variant else []) + [0, 0, 0, 0]
    sim = Simulation(resolved, kernel=DP_KERNEL_AUTO, device=device, cells_per_lane=v[0], tile_y=v[1],
                     ring_slots=v[2], z_chunk=v[3])
    sim.set_accumulate_intensity(True)
    stream = torch.cuda.ExternalStream(sim_stream(sim), device=device)
    cells = sim.cells

    def barrier():
        torch.cuda.synchronize(device)
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    sim.advance_by(args.regime)
    sim.wait(600_000)
    # The autotuner times each plan from this late-regime state (restoring it
    # exactly) and keeps the fastest for the timed window; untimed, like the
    # warm-up.
    tuned = None
    if not args.no_tune and not args.variant:
        tuned = sim.autotune(steps=8)
    sim.advance_by(args.warmup)
    sim.wait(600_000)
    barrier()
    first_timed = sim.step_count()
    start, end = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    launches0 = sim.launch_count()
    with ClockSampler(device) as clocks:
        start.record(stream)
        sim.advance_by(args.steps)
        end.record(stream)
        sim.wait(600_000)
        barrier()
    launches = sim.launch_count() - launches0
    plan = sim.plan()
    ms = max_over_ranks(start.elapsed_time(end), world)
    seconds = ms / 1e3
    value = world * cells * args.steps / seconds / 1e9

    # End to end through the public API, host buffers, copies inside the clock.
    e2e = None
    if not args.no_e2e:
        pinned_e = torch.empty(3 * cells, dtype=torch.float32, pin_memory=True)
        pinned_h = torch.empty(3 * cells, dtype=torch.float32, pin_memory=True)
        pinned_i = torch.empty(cells, dtype=torch.float32, pin_memory=True)
        from diaphane_gb300 import Snapshot
        # Set-up, like the allocation: the late-regime state the device-timed
        # window ended in is read into the pinned buffers (one copy each way
        # through the same calls also faults the freshly pinned pages in for
        # DMA: measured on GB300, the first copy into new pinned memory took
        # 0.14 s for 3.8 GB after a minute of CPU load, every later one
        # 0.02 s).  The timed run restores that state from the host and
        # steps the same regime again.
        sim.wait(600_000)
        snap_step = sim.step_count()
        # Two rounds: after the tests or other host load the first copies into
        # new pinned memory have measured up to 8x slower than later ones.
        for _ in range(2):
            read_into(sim, pinned_i, pinned_e, pinned_h)
            sim.restore(Snapshot(snap_step, pinned_e.numpy(), pinned_h.numpy()))
            sim.wait(600_000)
        barrier()
        t0 = time.perf_counter()
        sim.restore(Snapshot(snap_step, pinned_e.numpy(), pinned_h.numpy()))
        sim.set_accumulate_intensity(False)
        sim.set_accumulate_intensity(True)
        sim.advance_by(args.steps)
        read_intensity_into(sim, pinned_i)
        barrier()
        e2e_s = max_over_ranks(time.perf_counter() - t0, world)
        h2d = 24 * cells / args.steps
        d2h = 4 * cells / args.steps
        e2e = {"value": world * cells * args.steps / e2e_s / 1e9, "unit": "Gcell/s",
               "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "what": "inputs: the late-regime state E,H (step %d) restored from pinned host memory; advance K "
                       "steps accumulating intensity; result: the intensity read back into pinned host memory; "
                       "wall clock" % snap_step}

    # Every rank takes part in the batch measurement (its scenes, then the
    # slowest rank's time); the rest is rank 0's.
    kernel_name = ["", "fused", "naive"][sim.kernel]
    accuracy = None
    if rank == 0 and world == 1 and not args.no_accuracy:
        try:
            accuracy = default_accuracy(sim, resolved, device)
        except Exception as exc:  # reported, not fatal to the headline line
            accuracy = {"error": f"{type(exc).__name__}: {exc}"}
    sim.close()
    batched = None
    if not args.no_batched:
        try:
            batched = batched_measurement(args.scenes, args.batch_steps, device, rank, world)
        except Exception as exc:  # reported, not fatal to the headline line
            batched = {"error": f"{type(exc).__name__}: {exc}"}
    served = None
    if rank == 0 and world == 1 and not args.no_served:
        try:
            served = default_served(device, value)
        except Exception as exc:  # reported, not fatal to the headline line
            served = {"error": f"{type(exc).__name__}: {exc}"}
    if rank != 0:
        return
    peak, peak_kind = measured_peaks()
    achieved = BYTES_PER_CELL * cells / (seconds / args.steps) / 1e9
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": profiled_traffic(args.side), "peak_kind": peak_kind,
                "algorithmic_bytes_per_launch": BYTES_PER_CELL * cells,
                "note": "48 B/cell-update of field traffic; the u8 material index (1 B) and the "
                        "intensity read-modify-write (8 B) move on top of it"}
    cpu = None
    if world == 1 and not args.no_cpu:
        threads = os.cpu_count() or 1
        rate, steps, elapsed = cpu_port_rate(scene, threads, budget_s=12.0, max_steps=200, warmup=1)
        rate1, steps1, elapsed1 = cpu_port_rate(scene, 1, budget_s=8.0, max_steps=50, warmup=0)
        cpu = {"value": rate, "unit": "Gcell/s", "cores": threads, "kind": "port",
               "sample": f"{steps} oracle steps of the same {args.side}^3 scene after 1 untimed, {elapsed:.1f} s",
               "single_thread": {"value": rate1, "unit": "Gcell/s", "cores": 1,
                                 "sample": f"{steps1} oracle steps, {elapsed1:.1f} s"},
               "nproc": os.cpu_count(), "cpu_model": cpu_model()}
    line = {"metric": "Gcell-updates/s", "value": value, "unit": "Gcell/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded SplitMix64 scene)",
            "config": config(args.side, world), "kernel": kernel_name,
            "variant": args.variant or "default",
            "regime": {"timed_from_step": first_timed,
                       "what": f"{args.regime} untimed steps and {args.warmup} warm-up steps before the timed "
                               "window: the wave has crossed the box and the absorbers hold decaying field"},
            "plan": plan, "tuned": tuned,
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "gpu_launches": launches,
            "clocks": clocks.summary(), "batched": batched, "served": served, "accuracy": accuracy}
    print(json.dumps(line), flush=True)


def sim_stream(sim) -> int:
    import ctypes as C
    from diaphane_gb300 import _abi
    p = C.c_void_p()
    _abi.check(_abi.lib().dp_sim_stream(sim.handle, C.byref(p)))
    return p.value or 0


def read_intensity_into(sim, intensity) -> None:
    from diaphane_gb300 import _abi
    _abi.check(_abi.lib().dp_sim_read_field(sim.handle, _abi.DP_FIELD_INTENSITY, intensity.data_ptr(),
                                            intensity.numel()))


def read_into(sim, intensity, electric, magnetic) -> None:
    from diaphane_gb300 import _abi
    lib = _abi.lib()
    _abi.check(lib.dp_sim_read_field(sim.handle, _abi.DP_FIELD_INTENSITY, intensity.data_ptr(), intensity.numel()))
    _abi.check(lib.dp_sim_read_field(sim.handle, _abi.DP_FIELD_ELECTRIC, electric.data_ptr(), electric.numel()))
    _abi.check(lib.dp_sim_read_field(sim.handle, _abi.DP_FIELD_MAGNETIC, magnetic.data_ptr(), magnetic.numel()))


BATCH_SEED = 0xBA7C_0000


def batched_measurement(scene_count: int, steps: int, device: int = 0, rank: int = 0, world: int = 1) -> dict:
    """Mixed-size batch vs this project's plain one-scene-at-a-time solver.

    Scenes: axes log-uniform in [32, 160] cells, seeded spheres, an optional
    conductor, one point or plane-wave source each (workloads.mixed_scene).
    Host scene setup is done up front for both; each arm's clock covers
    allocation, upload, stepping and reading every scene's E field back into
    that arm's own slice of pinned host memory (the same read call in both
    arms).  After both clocks every scene's E field is compared bit for bit
    between the arms."""
    import numpy as np
    import torch
    from diaphane_gb300 import Batch, ResolvedScene, Simulation, workloads
    mine = partition(scene_count, rank, world)  # replicas split the scenes; nothing is exchanged
    resolved = [ResolvedScene(workloads.mixed_scene(BATCH_SEED + k)) for k in mine]
    cells = sum(ResolvedScene(workloads.mixed_scene(BATCH_SEED + k)).cells for k in range(scene_count)) \
        if world > 1 else sum(r.cells for r in resolved)
    offsets = np.cumsum([0] + [3 * r.cells for r in resolved])
    plain_out = torch.empty(int(offsets[-1]), dtype=torch.float32, pin_memory=True).numpy()
    batch_out = torch.empty(int(offsets[-1]), dtype=torch.float32, pin_memory=True).numpy()
    # Set-up, like the allocation: one device-to-host copy into each buffer
    # faults its freshly pinned pages in for DMA before either clock starts.
    scratch = torch.zeros(int(offsets[-1]), dtype=torch.float32, device=f"cuda:{device}")
    for host in (plain_out, batch_out, plain_out, batch_out):
        torch.from_numpy(host).copy_(scratch)
    del scratch
    torch.cuda.synchronize(device)
    # Plain: one Simulation per scene, one after another.
    t0 = time.perf_counter()
    for k, r in enumerate(resolved):
        sim = Simulation(r, device=device)
        sim.advance_by(steps)
        sim.read_electric(out=plain_out[offsets[k]:offsets[k + 1]])
        sim.close()
    plain_s = max_over_ranks(time.perf_counter() - t0, world)
    # The plain solver again with 32-wide tiles forced: its planner keeps the
    # widest tile that wastes no more lanes, and on these small grids the
    # narrowest measured as fast or faster for every scene sampled; this arm
    # is the stronger plain baseline, reported beside the default one.
    narrow_out = torch.empty(int(offsets[-1]), dtype=torch.float32, pin_memory=True).numpy()
    torch.from_numpy(narrow_out).copy_(torch.from_numpy(plain_out))
    t0 = time.perf_counter()
    for k, r in enumerate(resolved):
        sim = Simulation(r, device=device, cells_per_lane=1)
        sim.advance_by(steps)
        sim.read_electric(out=narrow_out[offsets[k]:offsets[k + 1]])
        sim.close()
    narrow_s = max_over_ranks(time.perf_counter() - t0, world)
    # Batched: one arena, one launch per step per kernel variant, K-step graphs.
    arena = int(1.05 * sum(Batch.bytes_for(r, steps) for r in resolved)) + (64 << 20)
    batch = Batch(arena, chunk_steps=50, max_scenes=max(1, len(resolved)), device=device)
    t0 = time.perf_counter()
    ids = [batch.add(r, steps) for r in resolved]
    batch.wait()
    t1 = time.perf_counter()
    batch.run_to_completion()
    t2 = time.perf_counter()
    for k, i in enumerate(ids):
        batch.read_electric(i, out=batch_out[offsets[k]:offsets[k + 1]])
    t3 = time.perf_counter()
    batched_s = max_over_ranks(t3 - t0, world)
    stepping_s = max_over_ranks(t2 - t1, world)
    identical = [bool(np.array_equal(batch_out[offsets[k]:offsets[k + 1]].view(np.uint32),
                                     plain_out[offsets[k]:offsets[k + 1]].view(np.uint32)) and
                      np.array_equal(narrow_out[offsets[k]:offsets[k + 1]].view(np.uint32),
                                     plain_out[offsets[k]:offsets[k + 1]].view(np.uint32)))
                 for k in range(len(resolved))]
    peak, peak_kind = measured_peaks()
    step_gbs = BYTES_PER_CELL * cells * steps / stepping_s / 1e9
    return {"scenes": scene_count, "steps": steps, "cells": cells,
            "phases_s": {"add": t1 - t0, "stepping": t2 - t1, "read": t3 - t2},
            "stepping_roofline": {"bound": "hbm", "achieved": step_gbs, "peak": peak, "unit": "GB/s",
                                  "frac": step_gbs / peak, "peak_kind": peak_kind,
                                  "what": "48 B per cell-update over the stepping phase's wall clock "
                                          "(graph replays, staging and launches included)"},
            "batched_solves_per_s": scene_count / batched_s, "plain_solves_per_s": scene_count / plain_s,
            "speedup": plain_s / batched_s, "batched_gcells": cells * steps / batched_s / 1e9,
            "plain_32wide_s": narrow_s, "speedup_vs_plain_32wide": narrow_s / batched_s,
            "plain_32wide_what": "the plain solver with cells_per_lane=1 forced for every scene (its planner "
                                 "picks the widest tile that wastes no more lanes; on these grids 32-wide "
                                 "tiles measured as fast or faster for every scene sampled)",
            "plain_gcells": cells * steps / plain_s / 1e9, "batched_s": batched_s, "plain_s": plain_s,
            "chunk_steps": 50, "graph_launches": batch.launch_count(),
            "bit_identical_to_plain": all(identical), "scenes_compared": len(identical),
            "scenes_identical": sum(identical), "replicas": world,
            "scaling": "strong (the 256 scenes are split across replicas)"}


def default_accuracy(sim, resolved, device: int) -> dict:
    """FP64 error of the configurations the line stands for, on the GPU:
    the metric's 512³ scene at the step this run ended on (the f32 fields of
    the benchmarked simulation against the FP64 instance stepped as far),
    free flight 80³ at 1000 steps normalized by the launched peak, the
    graded stack 640×256×256 at its 5000 steps, the 192³ graded conducting
    box's windowed energy drift over 20,000 steps in f32 and FP64, and a
    sample of the mixed-size batch's scenes (the served stream's scenes are
    drawn the same way) at 1000 steps."""
    from diaphane_gb300 import Simulation64, workloads
    steps = sim.step_count()
    f64 = Simulation64(resolved, device=device)
    f64.advance_by(steps)
    f64.wait(1_800_000)
    e32, e64 = sim.energy().total(), f64.energy().total()
    metric = {"case": WORKLOAD, "steps": steps,
              "E": field_error(sim.read_electric(), f64.read_electric()),
              "H": field_error(sim.read_magnetic(), f64.read_magnetic()),
              "energy_rel_diff": abs(e32 - e64) / e64 if e64 else None,
              "normalization": "max |f32 - f64| over all three components / max |f64| at that step"}
    f64.close()
    return {"heterogeneous_512": metric, "free_flight_80": free_flight_accuracy(device),
            "graded_stack": accuracy_case("graded stack 640x256x256", workloads.graded_stack(), 5000, device),
            "graded_cavity_drift": drift_case(device),
            "batched_sample": [accuracy_case(f"mixed scene {k}", workloads.mixed_scene(BATCH_SEED + k), 1000, device)
                               for k in range(3)]}


def free_flight_accuracy(device: int = 0, steps: int = 1000, every: int = 50) -> dict:
    """Free flight 80³: the f32 step and the FP64 instance side by side.  The
    packet leaves through the absorber, so the error is stated against the
    launched peak (the largest |E| of the FP64 run at any sampled step), at
    the end and at its worst over the run."""
    import numpy as np
    from diaphane_gb300 import ResolvedScene, Simulation, Simulation64, workloads
    resolved = ResolvedScene(workloads.free_flight(80))
    f32, f64 = Simulation(resolved, device=device), Simulation64(resolved, device=device)
    launched, worst, last = 0.0, 0.0, 0.0
    for _ in range(steps // every):
        f32.advance_by(every)
        f64.advance_by(every)
        a, b = f32.read_electric().astype(np.float64), f64.read_electric()
        launched = max(launched, float(np.abs(b).max()))
        last = float(np.abs(a - b).max())
        worst = max(worst, last)
    f32.close()
    f64.close()
    return {"case": "free flight 80^3", "steps": steps, "launched_peak": launched,
            "E_at_end_of_launched_peak": last / launched, "E_worst_of_launched_peak": worst / launched,
            "normalization": f"max |f32 - f64| of E / the largest |E| of the FP64 run, sampled every {every} steps"}


def default_served(device: int, plain_rate_gcells: float, rate: float = 16.0, count: int = 48) -> dict:
    """One Poisson trace (48 requests at 16/s) served by continuous batching
    and by the plain solver, with the ceilings that bound it: the trace's
    cell-updates at the single-scene 512³ rate, and the arrivals themselves."""
    results = served_measurement([rate], count, device)[0]
    from diaphane_gb300.serve import poisson_trace
    trace = poisson_trace(count, rate)
    cell_updates = 0
    work = []
    for r in trace:
        r.resolve()
        cell_updates += r.cells * r.steps
        work.append((r.arrival, r.cells * r.steps))
        r.resolved = None
    stepping_s = cell_updates / (plain_rate_gcells * 1e9)
    last_arrival = max(r.arrival for r in trace)
    # Work that arrives at or after time t cannot finish before t plus its
    # stepping time at the 512^3 rate: the largest such bound over t bounds
    # the makespan from below, whatever the scheduler.
    work.sort()
    first = work[0][0]
    makespan_bound = max(a - first + sum(w for _, w in work[i:]) / (plain_rate_gcells * 1e9)
                         for i, (a, _) in enumerate(work))
    results["ceiling"] = {
        "cell_updates": cell_updates,
        "stepping_s_at_512_rate": stepping_s,
        "solves_per_s_at_512_rate": count / stepping_s,
        "last_arrival_s": last_arrival,
        "what": "the trace's cell-updates at this run's plain 512^3 rate bound solves/s from above (the plain "
                "solver already runs its large requests near that rate); arrivals end at last_arrival_s"}
    results["ceiling"]["speedup_bound_over_plain"] = (count / stepping_s) / results["plain"]["solves_per_s"]
    results["ceiling"]["makespan_lower_bound_s"] = makespan_bound
    results["ceiling"]["solves_per_s_bound_with_arrivals"] = count / makespan_bound
    results["ceiling"]["speedup_bound_with_arrivals"] = (count / makespan_bound) / results["plain"]["solves_per_s"]
    results["ceiling"]["arrivals_what"] = (
        "work arriving at or after t cannot finish before t + its stepping time at the plain 512^3 rate; the "
        "largest such bound over t (from the first arrival) bounds the makespan of any schedule")
    return results


def run_batched(args):
    line = {"metric": "solves/s (batched mixed sizes)", "workload": "batched"}
    line.update(batched_measurement(args.scenes, args.batch_steps))
    line["value"] = line["batched_solves_per_s"]
    line["unit"] = "solves/s"
    print(json.dumps(line), flush=True)


def served_measurement(rates, count: int, device: int = 0, arena_bytes: int = 150 * 10**9) -> list:
    """Poisson arrival traces replayed twice each: continuous batching over
    one arena (admission by bytes, join and leave at 50-step chunk
    boundaries, 8 probes of Ez/Hy per step) and the plain solver, first come
    first served, recording the same probe series.  Scene axes log-uniform in
    [48, 320] cells, steps uniform in [200, 5000].  Latency = completion
    (results on the host) - arrival.  Every request's series is compared bit
    for bit between the two replays."""
    import numpy as np
    from diaphane_gb300.serve import Server, poisson_trace, serve_plain, summary
    server = Server(arena_bytes, max_scenes=256, chunk_steps=50, device=device)
    warm = dict(lo=48, hi=64, steps=(50, 60))
    server.serve(poisson_trace(2, 100.0, seed=1, **warm))
    serve_plain(poisson_trace(2, 100.0, seed=1, **warm), device)
    out = []
    for rate in rates:
        trace = server.serve(poisson_trace(count, rate))
        served = summary(trace)
        served["chunks"] = server.chunks
        served["peak_active"] = server.peak_active
        plain_trace = serve_plain(poisson_trace(count, rate), device)
        plain = summary(plain_trace)
        same = sum(bool(np.array_equal(a.series.view(np.uint32), b.series.view(np.uint32)))
                   for a, b in zip(sorted(trace, key=lambda r: r.ident), sorted(plain_trace, key=lambda r: r.ident)))
        out.append({"arrivals_per_s": rate, "served": served, "plain": plain,
                    "series_identical": same, "series_compared": len(trace),
                    "p99_ratio_plain_over_served": plain["p99_s"] / served["p99_s"],
                    "throughput_ratio": served["solves_per_s"] / plain["solves_per_s"]})
        server.chunks = 0
        server.peak_active = 0
    server.close()
    return out


def run_served(args):
    rates = [float(r) for r in args.rates.split(",")]
    results = served_measurement(rates, args.requests)
    top = results[-1]["served"]
    line = {"metric": "solves/s (served, Poisson arrivals)", "workload": "served", "value": top["solves_per_s"],
            "unit": "solves/s", "requests_per_trace": args.requests, "arena_bytes": 150 * 10**9,
            "scene_axes": [48, 320], "steps": [200, 5000], "probes": 8, "by_rate": results}
    print(json.dumps(line), flush=True)


def field_error(a32, b64, chunk: int = 1 << 24) -> dict:
    """f32 field against its FP64 counterpart: max |difference| as a
    fraction of the FP64 peak, and the relative L2 norm."""
    import numpy as np
    peak = worst = sd = sb = 0.0
    for i in range(0, b64.size, chunk):
        y = b64[i:i + chunk]
        d = a32[i:i + chunk].astype(np.float64) - y
        worst = max(worst, float(np.abs(d).max()))
        peak = max(peak, float(np.abs(y).max()))
        sd += float(np.dot(d, d))
        sb += float(np.dot(y, y))
    return {"max_abs_over_peak": worst / peak if peak else None, "rel_l2": (sd / sb) ** 0.5 if sb else None,
            "peak": peak}


def accuracy_case(name: str, scene, steps: int, device: int = 0) -> dict:
    """The product's f32 step against the FP64 instance on the GPU, same
    scene, same step count."""
    from diaphane_gb300 import ResolvedScene, Simulation, Simulation64
    resolved = ResolvedScene(scene)
    f32 = Simulation(resolved, device=device)
    f64 = Simulation64(resolved, device=device)
    t0 = time.perf_counter()
    f32.advance_by(steps)
    f32.wait(600_000)
    t32 = time.perf_counter() - t0
    t0 = time.perf_counter()
    f64.advance_by(steps)
    f64.wait(1_800_000)
    t64 = time.perf_counter() - t0
    e32, e64 = f32.energy().total(), f64.energy().total()
    out = {"case": name, "extent": list(resolved.extent), "steps": steps,
           "E": field_error(f32.read_electric(), f64.read_electric()),
           "H": field_error(f32.read_magnetic(), f64.read_magnetic()),
           "energy_rel_diff": abs(e32 - e64) / e64 if e64 else None,
           "f32_kernel": ["", "fused", "naive"][f32.kernel], "f32_s": t32, "f64_s": t64}
    f32.close()
    f64.close()
    return out


def drift_case(device: int = 0, early: int = 400, late: int = 20_000, window: int = 200) -> dict:
    """Windowed-mean energy drift of the 192³ graded conducting box: mean
    total energy over `window` steps after `early` steps, again after `late`
    more, for the f32 step and the FP64 instance."""
    from diaphane_gb300 import ResolvedScene, Simulation, Simulation64, workloads
    resolved = ResolvedScene(workloads.graded_cavity())

    def mean_energy(sim):
        total = 0.0
        for _ in range(window):
            sim.advance_by(1)
            total += sim.energy().total()
        return total / window

    out = {"case": "graded cavity (PEC)", "extent": list(resolved.extent), "early": early, "late": late,
           "window": window}
    for name, sim in (("f32", Simulation(resolved, device=device)), ("f64", Simulation64(resolved, device=device))):
        sim.advance_by(early)
        a = mean_energy(sim)
        sim.advance_by(late)
        b = mean_energy(sim)
        out[f"drift_{name}"] = abs(b - a) / a
        sim.close()
    return out


def extras_measurement(side: int = 256, device: int = 0) -> dict:
    """The costs of the paths around the step, on the heterogeneous scene:
    scene rasterization (device against host), a backward scrub with the
    keyframes in device memory against keyframes on the host, a rendered
    frame, and the probe gather's per-step cost.  Wall clock, synchronized."""
    import numpy as np
    import torch
    from diaphane_gb300 import DeviceTimeline, ResolvedScene, Simulation, Timeline, _abi, workloads
    from diaphane_gb300.render import Renderer, View
    out = {"side": side}
    scene = workloads.heterogeneous(side)
    resolved = ResolvedScene(scene)
    # Rasterization: the u8 index on the device vs the host rasterizer (all cores).
    buf = torch.empty(resolved.cells, dtype=torch.uint8, device=f"cuda:{device}")
    resolved.rasterize(buf.data_ptr())
    torch.cuda.synchronize(device)
    t0 = time.perf_counter()
    for _ in range(5):
        resolved.rasterize(buf.data_ptr())
    torch.cuda.synchronize(device)
    device_ms = (time.perf_counter() - t0) / 5 * 1e3
    t0 = time.perf_counter()
    host = ResolvedScene(scene).table(_abi.DP_TABLE_MATERIAL_INDEX)
    host_ms = (time.perf_counter() - t0) * 1e3
    out["raster"] = {"device_ms": device_ms, "host_ms_including_setup": host_ms, "host_threads": os.cpu_count(),
                     "identical": bool(np.array_equal(buf.cpu().numpy(), host)), "shapes": len(scene.shapes)}
    del buf
    # Scrubbing: 10 keyframes 20 steps apart, then seeks back to 15 targets.
    sims = {}
    for kind in ("device", "host"):
        sim = Simulation(resolved, device=device)
        tl = DeviceTimeline(sim, 20, 10) if kind == "device" else Timeline(20, 10)
        for _ in range(40):
            sim.advance_by(5)
            tl.observe(sim)
        sim.wait()
        # Each target lies one step past a keyframe and below the last one,
        # so every seek restores a keyframe and replays a single step.
        targets = [181, 161, 141, 121, 101, 81, 61, 41, 21]
        t0 = time.perf_counter()
        for target in targets:
            outcome = tl.seek(sim, target)
            assert outcome.kind == "keyframe" and outcome.replayed == 1, outcome
            sim.wait()
        seek_ms = (time.perf_counter() - t0) / len(targets) * 1e3
        sims[kind] = (sim, tl)
        out[f"scrub_{kind}_keyframes_ms"] = seek_ms
    out["scrub_note"] = ("mean wall time of 9 backward seeks, each restoring a keyframe and replaying one "
                         "step; keyframes every 20 steps, 24 B per cell each")
    same = np.array_equal(sims["device"][0].read_electric().view(np.uint32),
                          sims["host"][0].read_electric().view(np.uint32))
    out["scrub_identical"] = bool(same)
    sim, device_timeline = sims["device"]
    del sims
    # A frame of the E-and-H view at 1280x720.
    renderer = Renderer(sim, 1280, 720)
    renderer.measure()
    renderer.draw(View())
    sim.wait()
    t0 = time.perf_counter()
    for k in range(10):
        renderer.draw(View(yaw=0.9 + 0.05 * k))
    sim.wait()
    out["render_ms_per_frame"] = (time.perf_counter() - t0) / 10 * 1e3
    out["render_size"] = [1280, 720]
    # Probes: 8 cells recorded every step.
    stream = torch.cuda.ExternalStream(sim_stream(sim), device=device)
    def timed(steps):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        sim.advance_by(steps)
        b.record(stream)
        sim.wait()
        return a.elapsed_time(b) / steps
    # The same 60 steps from the same keyframe, without and then with probes.
    device_timeline.seek(sim, 100)
    plain = timed(60)
    device_timeline.seek(sim, 100)
    sim.set_probes([(side // 2, side // 2, k * side // 8) for k in range(8)], 1024)
    probed = timed(60)
    out["probe_us_per_step"] = (probed - plain) * 1e3
    out["step_ms"] = plain
    return out


def kernels_measurement(side: int = 256, device: int = 0) -> dict:
    """Every kernel around the fused step, a few launches each on the
    heterogeneous scene at side³, for a launch list with DRAM counters: the
    rasterizer, the one-thread-per-cell passes (H, E, each injection,
    intensity) in f32 and in f64, the energy, finiteness and energy-density
    reductions, the probe gather, row packing for a grid whose rows are
    padded, the renderer's reduction and ray march, and the batch's probe
    gather.  Wall times are reported; the per-kernel figures come from ncu."""
    import torch
    from diaphane_gb300 import (DP_KERNEL_NAIVE, Batch, ResolvedScene, Simulation, Simulation64, workloads)
    from diaphane_gb300.render import Renderer
    t0 = time.perf_counter()
    resolved = ResolvedScene(workloads.heterogeneous(side))
    index = torch.empty(resolved.cells, dtype=torch.uint8, device=f"cuda:{device}")
    resolved.rasterize(index.data_ptr())
    sim = Simulation(resolved, kernel=DP_KERNEL_NAIVE, device=device)
    sim.set_accumulate_intensity(True)
    sim.set_probes([(side // 2, side // 2, k * side // 8) for k in range(8)], 64)
    sim.advance_by(3)
    sim.energy()
    sim.is_finite()
    sim.energy_density()
    renderer = Renderer(sim, 1280, 720)
    renderer.measure()
    renderer.draw()
    sim.wait()
    renderer.close()
    sim.close()
    fp64 = Simulation64(resolved, device=device)
    fp64.advance_by(2)
    fp64.energy()
    fp64.close()
    odd = ResolvedScene(workloads.heterogeneous(side - 2))  # rows padded from side-2 to side cells
    padded = Simulation(odd, device=device)
    padded.advance_by(2)
    padded.write_electric(padded.read_electric())
    padded.close()
    small = [ResolvedScene(workloads.mixed_scene(BATCH_SEED + k)) for k in range(4)]
    batch = Batch(int(1.05 * sum(Batch.bytes_for(r, 4) for r in small)) + (64 << 20), chunk_steps=4,
                  max_scenes=4, device=device)
    for r in small:
        batch.add(r, 4, probes=[(4, 4, 4), (8, 8, 8)])
    batch.run_to_completion()
    batch.close()
    torch.cuda.synchronize(device)
    return {"side": side, "seconds": time.perf_counter() - t0}


def run_accuracy(args):
    from diaphane_gb300 import workloads
    cases = [accuracy_case("heterogeneous 512^3", workloads.heterogeneous(512), 2000),
             accuracy_case("graded stack 640x256x256", workloads.graded_stack(), 5000)]
    cases += [accuracy_case(f"mixed scene {k}", workloads.mixed_scene(BATCH_SEED + k), 1000) for k in range(8)]
    line = {"metric": "f32 error against the FP64 instance", "workload": "accuracy", "cases": cases,
            "free_flight": free_flight_accuracy(), "drift": drift_case()}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "batched":
        run_batched(args)
    elif args.workload == "served":
        run_served(args)
    elif args.workload == "accuracy":
        run_accuracy(args)
    elif args.workload == "extras":
        line = {"metric": "costs around the step", "workload": "extras"}
        line.update(extras_measurement(args.side if args.side != 512 else 256))
        print(json.dumps(line), flush=True)
    elif args.workload == "kernels":
        line = {"metric": "every kernel around the fused step, for ncu", "workload": "kernels"}
        line.update(kernels_measurement(args.side if args.side != 512 else 256))
        print(json.dumps(line), flush=True)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
