"""The multi-GPU path of bench.py on CPU: two gloo ranks (replicas) with
unequal work and times; the whole-job throughput is the sum of the ranks'
paths over the slowest rank's time, the same on every rank."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    paths = [100e6, 120e6][rank]
    rays = [400e6, 500e6][rank]
    ms = [1000.0, 1500.0][rank]
    q.put((rank, bench.aggregate(dist, paths, rays, ms, "cpu")))
    dist.barrier()
    dist.destroy_process_group()


def test_replicas_aggregate_over_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in range(2):
        mpaths, mrays, ms = got[r]
        assert ms == pytest.approx(1500.0)
        assert mpaths == pytest.approx(220e6 / 1.5 / 1e6)
        assert mrays == pytest.approx(900e6 / 1.5 / 1e6)


def test_single_process_aggregate():
    import bench
    assert bench.aggregate(None, 50e6, 200e6, 500.0) == pytest.approx((100.0, 400.0, 500.0))
