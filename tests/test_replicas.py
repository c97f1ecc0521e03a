"""The N > 1 path of bench.py on CPU: torchrun launches one rank per GPU, each
running an independent replica of the step (no data-path collective); the
job's time is the slowest rank's and its rate counts every replica's cells.
Checked with world_size 2 over gloo, with the helpers bench.py uses; the
reference arm runs on rank 0 only and the other ranks exit without output.
"""
import io
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # ranks time different durations: the job takes the slowest
        ms = [3.0, 5.0][rank]
        ms_max = bench.max_over_ranks(ms, dist, "cpu")
        rate = bench.whole_job_rate(2048 * 2048 * 100, world, ms_max * 1e-3)
        # the reference arm: only rank 0 may print
        buf = io.StringIO()

        class Args:
            steps, warmup = 1, 0
        with redirect_stdout(buf):
            if rank != 0:
                bench.run_reference(Args(), rank)
        q.put((rank, ms_max, rate, buf.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_replicas_over_gloo():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    out.sort()
    for rank, ms_max, rate, printed in out:
        assert ms_max == 5.0
        assert rate == 2 * 2048 * 2048 * 100 / 5e-3
        assert printed == ""


def test_single_rank_helpers():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(4.5) == 4.5
    assert bench.whole_job_rate(10.0, 1, 2.0) == 5.0


def test_checkpoints_of_the_error_curves():
    sys.path.insert(0, REPO)
    import bench
    assert bench.checkpoints(800) == [100, 200, 300, 400, 500, 600, 700, 800]
    assert bench.checkpoints(3) == [1, 2, 3]
    pts = bench.checkpoints(1637)
    assert pts[-1] == 1637 and len(pts) == 8 and pts == sorted(set(pts))
