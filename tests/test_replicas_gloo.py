"""The multi-GPU form of the benchmark is replicas only (independent problems per rank, no data-
path collective): its rank logic -- the slowest rank's time, the whole-job rate, and the
reference arm running on rank 0 alone -- checked with world_size 2 over gloo on the CPU."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 * (rank + 1), dist, "cpu")
    rate = bench.aggregate_rate(1, 5, ms, world)
    dist.destroy_process_group()
    q.put((rank, ms, rate))


def test_max_over_ranks_and_rate_gloo():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # both ranks see the slowest rank's 20 ms; 2 ranks x 5 steps / 20 ms = 500 iterations/s
    assert [g[1] for g in got] == [20.0, 20.0]
    assert all(abs(g[2] - 500.0) < 1e-9 for g in got)


def test_reference_arm_runs_on_rank0_only():
    """Under a 2-rank launch the reference arm's rank 1 exits 0 without work or output."""
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "3"], capture_output=True, text=True,
                       timeout=120, env=env)
    assert r.returncode == 0 and r.stdout.strip() == ""
