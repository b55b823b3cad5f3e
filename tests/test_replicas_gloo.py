"""The multi-GPU form of the bench is replicas only (the path has no data
exchange between cases): each rank times its own replica, the job time is the
slowest rank's and the rate counts every rank's cells.  The reduction runs
here as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

import bench


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [120.0, 150.0][rank]
    worst = bench.reduce_max(dist, ms, "cpu")
    q.put((rank, worst, bench.aggregate_rate(18432, 10, world, worst)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    res = sorted(q.get(timeout=5) for _ in range(2))
    assert [r[1] for r in res] == [150.0, 150.0]
    assert res[0][2] == pytest.approx(18432 * 10 * 2 / 0.150)


def test_single_process_reduction_is_identity():
    assert bench.reduce_max(None, 3.5, "cpu") == 3.5
