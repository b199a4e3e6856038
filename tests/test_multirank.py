"""Replicas across ranks (bench.py --gpus N): the whole-job figure is the
sum of the ranks' work over the slowest rank's time.  Two gloo ranks on CPU."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units = 1000.0 * (rank + 1)          # rank 0: 1000, rank 1: 2000
    seconds = 2.0 if rank == 1 else 1.0  # rank 1 is the slowest
    v, t = bench.reduce_replicas(units, seconds, dist)
    q.put((rank, v, t))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_reduction_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, v, t in res:
        assert t == 2.0
        assert v == pytest.approx(3000.0 / 2.0)


def test_single_rank_without_process_group():
    import bench
    v, t = bench.reduce_replicas(500.0, 0.5, None)
    assert v == 1000.0 and t == 0.5
