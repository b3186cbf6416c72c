"""Replicas (the only multi-GPU form of this path: tiles are independent, no
collective on the data path): the bench's whole-job rate is all ranks'
pixels over the slowest rank's time.  Exercised here with two gloo ranks on
the CPU."""
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
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, ROOT)
    import bench
    ms_local = [1000.0, 2500.0][rank]  # rank 1 is the slow one
    value, ms = bench.replica_rate(1_000_000, ms_local, world)
    q.put((rank, value, ms))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_rate_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, ms in got:
        assert ms == 2500.0                      # the slowest rank's time on every rank
        assert value == pytest.approx(2 * 1_000_000 / 2.5 / 1e6)  # both ranks' pixels


def test_replica_rate_single_rank():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_rate(2_000_000, 500.0, 1) == (4.0, 500.0)
