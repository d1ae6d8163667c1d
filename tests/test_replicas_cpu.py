"""Multi-replica plumbing of bench.py on CPU: two gloo ranks on 127.0.0.1.

bench.py --gpus N runs N independent replicas (no data-path collective); the
only cross-rank steps are a barrier and a max over the ranks' timed regions.
These tests run that plumbing without a GPU: the whole-job rate is the units
all ranks processed over the slowest rank's time, and the reference arm does
its work on rank 0 only.
"""
import io
import json
import os
import socket
import sys
from contextlib import redirect_stdout

import pytest

torch = pytest.importorskip("torch")
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, out):
    os.environ.update({"WORLD_SIZE": str(world), "RANK": str(rank), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    sys.path.insert(0, ROOT)
    import bench
    d = bench.Dist()
    try:
        d.barrier()
        # rank r "took" 1 + r seconds for 1000 units
        rate, t = bench.replica_rate(1000.0, 1.0 + rank, d)
        buf = io.StringIO()
        with redirect_stdout(buf):
            if rank != 0:
                bench.run_reference(object(), d)  # must return before reading any argument
        out.put((rank, rate, t, buf.getvalue()))
    finally:
        d.close()


def test_two_gloo_ranks_rate_and_rank0_only_reference():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, rate, t, printed in res:
        assert t == pytest.approx(2.0)             # slowest rank
        assert rate == pytest.approx(2 * 1000.0 / 2.0)
        if rank != 0:
            assert printed == ""


def test_single_process_rate():
    sys.path.insert(0, ROOT)
    import bench
    for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK"):
        os.environ.pop(k, None)
    d = bench.Dist()
    rate, t = bench.replica_rate(500.0, 0.25, d)
    assert (rate, t) == (2000.0, 0.25)
    json.dumps({"rate": rate})
