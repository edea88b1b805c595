"""The replica path of bench.py for N > 1 on CPU: two gloo ranks (127.0.0.1) exercise what the GPU
run does with NCCL between replicas: the rank environment, the barrier around the timed region, the
job time as the slowest rank's, the whole-job value, and the reference arm doing no work off rank 0.
Each rank runs its own replica (no collective on the data path), so these are the only exchanges."""
import contextlib
import io
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch
    import torch.distributed as dist

    import bench

    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        w, r, local = bench.dist_setup()
        barrier, max_over_ranks = bench.rank_ops(torch, dist, "cpu")
        barrier()
        t = max_over_ranks(0.5 + rank)  # the replicas' own times; rank 1 is the slowest
        value = bench.job_value(w, 1000.0, t)
        out = io.StringIO()
        if r != 0:  # the reference arm: ranks other than 0 return at once and print nothing
            with contextlib.redirect_stdout(out):
                bench.run_reference(None, w, r)
        barrier()
        q.put((r, w, local, t, value, out.getvalue()))
    finally:
        dist.destroy_process_group()


def test_two_gloo_replica_ranks():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    try:
        res = sorted(q.get(timeout=180) for _ in procs)
    finally:
        for p in procs:
            p.join(timeout=60)
            if p.is_alive():
                p.kill()
    assert [p.exitcode for p in procs] == [0, 0]
    assert [r[:3] for r in res] == [(0, 2, 0), (1, 2, 1)]
    assert all(r[3] == pytest.approx(1.5) for r in res)  # every rank sees the slowest rank's time
    assert all(r[4] == pytest.approx(2 * 1000.0 / 1.5) for r in res)  # all units over that time
    assert res[1][5] == ""
