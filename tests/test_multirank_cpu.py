"""The cross-rank step of bench.py on two gloo ranks (CPU): each rank fits its own stamps;
the job's time is the slowest rank's and the fit counts add up."""

import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import torch.distributed as dist

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    res = bench.aggregate_ranks(100.0 + 50.0 * rank, 120.0 + 10.0 * rank, 90 + rank, 100, "cpu")
    out[rank] = res
    dist.destroy_process_group()


def test_two_rank_aggregation():
    ctx = torch.multiprocessing.get_context("spawn")
    port = _free_port()
    with ctx.Manager() as mgr:
        out = mgr.dict()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        for r in range(2):
            dev_ms, e2e_ms, conv, total = out[r]
            assert dev_ms == 150.0 and e2e_ms == 130.0
            assert conv == 181 and total == 200


def test_single_process_passthrough():
    import bench

    assert bench.aggregate_ranks(1.0, 2.0, 3, 4, "cpu") == (1.0, 2.0, 3, 4)
