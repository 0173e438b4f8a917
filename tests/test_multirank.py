"""The multi-GPU form on the CPU: replicas only.  Ranks run as gloo
processes on 127.0.0.1; the bench's reduction of the timed region (the
slowest rank's time), its split of independent scenes across replicas, and
the reference arm's rank-0-only line are checked without a GPU."""
import json
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, queue):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, str(ROOT))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", init_method="env://", rank=rank, world_size=world)
    slowest = bench.max_over_ranks(1.5 * (rank + 1), world)
    mine = bench.partition(11, rank, world)
    dist.barrier()
    dist.destroy_process_group()
    queue.put((rank, slowest, mine))


def test_two_replicas_agree_on_the_slowest_time_and_split_the_scenes():
    ctx = mp.get_context("spawn")
    queue = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, queue)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(queue.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in results] == [3.0, 3.0]
    shares = [set(r[2]) for r in results]
    assert shares[0].isdisjoint(shares[1]) and shares[0] | shares[1] == set(range(11))


def test_one_process_is_its_own_world():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(2.5, 1) == 2.5
    assert bench.partition(4, 0, 1) == [0, 1, 2, 3]


def test_the_reference_arm_prints_one_line_on_rank_zero_only():
    lines = {}
    for rank in (0, 1):
        env = dict(os.environ, RANK=str(rank), WORLD_SIZE="2", LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1")
        out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--side", "24", "--steps", "4",
                              "--warmup", "1", "--ref-budget", "2"], cwd=ROOT, env=env, capture_output=True,
                             text=True, timeout=300)
        assert out.returncode == 0, out.stderr[-2000:]
        lines[rank] = [l for l in out.stdout.splitlines() if l.strip()]
    assert lines[1] == []
    assert len(lines[0]) == 1
    line = json.loads(lines[0][0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
