"""The benchmark's multi-GPU bookkeeping (replicas: one model per rank, no
collective on the data path) on CPU with two gloo ranks: the slowest rank's
time is every rank's, and the whole-job throughput is all ranks' units over
it."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    value, t = bench._replica_throughput(100.0, 1.0 + rank, "cpu")
    out[rank] = (value, t, bench._max_over_ranks(10.0 * rank, "cpu"))
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    torch = pytest.importorskip("torch")
    mp = torch.multiprocessing.get_context("spawn")
    with mp.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [mp.Process(target=_worker, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    for r in range(2):
        value, t, mx = res[r]
        assert t == 2.0  # the slower rank's time on every rank
        assert value == pytest.approx(2 * 100.0 / 2.0)
        assert mx == 10.0


def test_single_process_is_its_own_max():
    pytest.importorskip("torch")
    sys.path.insert(0, ROOT)
    import bench

    assert bench._max_over_ranks(3.5, "cpu") == 3.5
    assert bench._replica_throughput(10.0, 2.0, "cpu") == (5.0, 2.0)
