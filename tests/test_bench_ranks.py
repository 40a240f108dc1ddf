"""The bench's multi-rank logic on the CPU (replicas only: no data-path
collective): two gloo ranks reduce their timings to the slowest rank's, the
whole-job rate counts every rank's units over that time, and the reference
arm runs on rank 0 alone."""
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


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    times = [100.0 + 10 * rank, 250.0 - 50 * rank]  # ranks differ; each entry's max is on a different rank
    out = bench.max_over_ranks(times, "cpu", world)
    dist.destroy_process_group()
    q.put((rank, out))


def test_timings_reduce_to_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[0] == res[1] == [110.0, 250.0]


def test_job_rate_counts_every_rank():
    sys.path.insert(0, ROOT)
    import bench
    # 2 ranks x 3 steps x 1e9 units in 1.5 s (the slowest rank)
    assert bench.job_rate(1e9, 3, 2, 1500.0) == pytest.approx(4e9)
    assert bench.job_rate(1e9, 3, 1, 1500.0) == pytest.approx(2e9)


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                        "--warmup", "0"], capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
