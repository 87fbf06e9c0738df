"""The N>1 path of bench.py is replicas only: each rank evolves its own
instance and only the timing/throughput scalars are combined (max of the
elapsed times, sum of the point-updates).  Checked here with two gloo ranks
on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import bench
    w, r, local, pg = bench.dist_setup(None)
    assert (w, r, local) == (world, rank, rank)
    elapsed = [3.0, 5.0][rank]
    updates = [1e6, 2e6][rank]
    mx = bench.max_over_ranks(pg, elapsed)
    tot = bench.sum_over_ranks(pg, updates)
    bench.barrier(pg)
    q.put((rank, mx, tot))
    dist.destroy_process_group()


def test_two_rank_aggregation():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = sorted(q.get(timeout=10) for _ in range(2))
    for rank, mx, tot in res:
        assert mx == 5.0 and tot == 3e6


def _ref_worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import io
    import contextlib
    import bench

    class A:
        gpus, steps, warmup = 2, 1, 0
    buf = io.StringIO()
    if rank != 0:
        with contextlib.redirect_stdout(buf):
            bench.run_reference(A())
        q.put((rank, buf.getvalue()))
    else:
        # rank 0 would time the CPU sample; here it only joins the group
        bench.dist_setup(A())
        q.put((rank, "rank0"))
    dist.destroy_process_group()


def test_reference_arm_other_ranks_exit_without_work():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_ref_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    res = dict(q.get(timeout=10) for _ in range(2))
    assert res[1] == ""
