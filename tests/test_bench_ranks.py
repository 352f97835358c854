"""The multi-rank logic of bench.py, on the CPU with two gloo ranks.  On a GPU node every
rank steps its own replica of the system (no exchange step); the ranks meet only for the
timing barrier and two reductions: the slowest rank's time (max) and the particles of all
ranks (sum), whose ratio is the whole-job particle-steps/s.  The reference arm runs on
rank 0 alone and the other ranks exit without work."""
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket(socket.AF_INET, socket.SOCK_STREAM) as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    w, r, local, dist = bench.dist_setup("gloo")
    bench.barrier(dist, local)
    slowest = bench.reduce_op(dist, 2.0 + r, "max")           # rank times 2 ms and 3 ms
    particles = bench.reduce_op(dist, 1000.0 * (r + 1), "sum")  # 1000 and 2000 particles
    value = bench.job_value(dist, 1000 * (r + 1), 5, 2.0 + r)
    bench.barrier(dist, local)
    dist.destroy_process_group()
    q.put((r, w, slowest, particles, value))


def test_two_ranks_reduce_like_the_benchmark():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = sorted(q.get(timeout=300) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r for r, *_ in results] == [0, 1]
    for _, world, slowest, particles, value in results:
        assert world == 2
        assert slowest == 3.0
        assert particles == 3000.0
        assert value == pytest.approx(3000.0 * 5 / 3.0e-3)  # all particles over the slowest rank


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3"],
                       cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
