"""Multi-GPU form: independent replicas (world_size 2 on gloo, CPU only).

bench.py aggregates replicas as the sum of every rank's solves over the
slowest rank's time; here two ranks report different work and times."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, world, port, q):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    secs, solves = (2.0, 32) if rank == 0 else (4.0, 16)
    q.put((rank, bench.replica_throughput(secs, solves, device="cpu")))
    dist.destroy_process_group()


def test_replica_throughput_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = dict(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for r in (0, 1):
        value, secs, solves = out[r]
        assert secs == 4.0 and solves == 48.0
        assert value == pytest.approx(12.0)


def test_replica_throughput_single_process():
    sys.path.insert(0, ROOT)
    import bench

    assert bench.replica_throughput(2.0, 10, device="cpu") == (5.0, 2.0, 10)
