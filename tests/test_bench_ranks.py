"""The benchmark's multi-rank host logic on CPU with two gloo ranks: the whole-job time is the
slowest rank's and the units are summed over ranks; the reference arm runs on rank 0 only."""
import os
import socket
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        ms = [10.0, 12.5][rank]
        units = [1000, 3000][rank]
        q.put((rank, bench.job_totals(ms, units, world, "cpu")))
    finally:
        dist.destroy_process_group()


def test_job_totals_two_gloo_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    out = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert out[0] == out[1] == (12.5, 4000.0)


def test_job_totals_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.job_totals(7.0, 11, 1, "cpu") == (7.0, 11)


def test_reference_arm_rank1_exits_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1",
                        "--warmup", "3"], cwd=ROOT, env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
