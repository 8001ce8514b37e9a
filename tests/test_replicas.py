"""Replica (N > 1) logic of bench.py on CPU: two gloo ranks agree on the
slowest rank's time and the whole-job rate; the reference arm runs on rank 0
only and other ranks exit 0 without output."""
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
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    ms = bench.max_over_ranks(10.0 + 5.0 * rank, world, device="cpu")
    rate = bench.aggregate_rate(world, 100, ms)
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, ms, rate))


def test_two_gloo_ranks_agree_on_max_time_and_job_rate():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    # Both ranks see the slowest rank's 15 ms; 2 ranks x 100 frames in 15 ms.
    for rank, ms, rate in got:
        assert ms == 15.0
        assert abs(rate - 200 / 0.015) < 1e-6


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(12.5, 1) == 12.5
    assert bench.aggregate_rate(1, 50, 100.0) == 500.0


def test_reference_arm_other_ranks_exit_quietly():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    p = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2"],
                       capture_output=True, text=True, env=env, timeout=300)
    assert p.returncode == 0
    assert p.stdout.strip() == ""
