"""Replica mode of bench.py on CPU ranks (gloo, world size 2).

The path runs on one GPU per process with no exchange between replicas;
the only cross-rank steps are the barrier and the max-over-ranks of the
step time, checked here without a GPU.
"""
import contextlib
import io
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [12.5, 31.0][rank]
    dist.barrier()
    m = bench.max_over_ranks(ms, dist, "cpu")
    v = bench.replica_throughput(1000, world, m)
    out.put((rank, m, v))
    dist.destroy_process_group()


def test_max_over_ranks_gloo_world2():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [31.0, 31.0]
    assert res[0][2] == pytest.approx(2 * 1000 / 31.0e-3)


def test_single_rank_passthrough():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(7.0, None, "cpu") == 7.0


def test_reference_arm_prints_only_on_rank0():
    sys.path.insert(0, ROOT)
    import bench

    class A:
        steps, warmup, gpus = 1, 1, 2
    buf = io.StringIO()
    with contextlib.redirect_stdout(buf):
        bench.run_reference_arm(A, rank=1)
    assert buf.getvalue() == ""
