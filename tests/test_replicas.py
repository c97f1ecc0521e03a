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


def test_binary32_rounded_state_matches_the_stored_conservative_state():
    import numpy as np
    sys.path.insert(0, REPO)
    import bench
    rng = np.random.default_rng(5)
    q = np.stack([rng.uniform(0.1, 2.0, (6, 7)), rng.uniform(-1, 1, (6, 7)), rng.uniform(-1, 1, (6, 7)),
                  rng.uniform(0.1, 3.0, (6, 7))], axis=-1)
    g = 1.4
    q2 = bench.binary32_rounded_state(q, g)

    def cons(x):
        r, u, v, p = (x[..., k] for k in range(4))
        return np.stack([r, r * u, r * v, p / (g - 1.0) + 0.5 * r * (u * u + v * v)], axis=-1)
    # the conservative state of the result is the binary32 rounding of q's
    assert np.allclose(cons(q2), cons(q).astype(np.float32).astype(np.float64), rtol=1e-13, atol=1e-15)
    assert np.array_equal(q2[..., 0], q[..., 0].astype(np.float32).astype(np.float64))
    rel = np.abs(q2 - q) / np.maximum(np.abs(q), 1e-30)
    assert 0 < rel.max() < 1e-6
