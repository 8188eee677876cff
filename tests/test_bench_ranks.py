"""bench.py's multi-rank logic on the CPU (gloo, world size 2): the job's
time is the max over ranks, only rank 0 reports, and the reference arm does
its work on rank 0 alone.  The GPU ranks are independent replicas (no
data-path collective), so this is all there is to shard."""
import io
import os
import contextlib
import socket

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(ws), LOCAL_RANK=str(rank))
    import torch.distributed as dist
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    got = bench.reduce_max(10.0 + 5.0 * rank)
    assert bench.dist_init() == (ws, rank, rank)

    class A:
        steps, warmup = 1, 0
    out = io.StringIO()
    if rank != 0:
        with contextlib.redirect_stdout(out):
            bench.run_reference(A())  # rank != 0: no work, no output
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, got, out.getvalue()))


def test_max_over_ranks_and_rank0_reporting():
    ws, port = 2, _free_port()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank, args=(r, ws, port, q)) for r in range(ws)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in range(ws))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [15.0, 15.0]
    assert res[1][2] == ""


def test_single_process_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5) == 3.5
