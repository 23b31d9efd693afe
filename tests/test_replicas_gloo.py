"""Replica bookkeeping of bench.py across ranks (world_size 2, gloo on CPU).

bench.py runs one independent replica per GPU with no data-path collective:
every rank solves its own work, and rank 0 reports the whole-job throughput
(sum of the units over the max of the per-rank times).  These tests run that
host logic in two CPU processes.
"""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    r, w, local = bench.dist_env()
    d = bench.Dist(w, local, backend="gloo")
    mv = 100.0 * (rank + 1)      # units this replica processed
    t = 0.5 + 0.25 * rank        # its timed region (s)
    d.barrier()
    t_max = d.max(t)
    mv_all = d.sum(mv)
    d.close()
    out.put((rank, t_max, mv_all, mv_all / t_max))


def test_two_replicas_report_sum_over_max():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t_max, mv_all, value in res:
        assert t_max == 0.75
        assert mv_all == 300.0
        assert value == 400.0


def _ref_worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench

    class Args:
        steps, warmup, gpus = 1, 0, world

    if rank != 0:  # only rank 0 times the CPU reference; the others leave at once
        out.put((rank, bench.reference_arm(Args, rank, world)))
    else:
        out.put((rank, None))


def test_reference_arm_runs_on_rank_zero_only():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_ref_worker, args=(r, 2, _free_port(), q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert res[1] == 0
