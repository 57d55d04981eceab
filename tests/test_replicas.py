"""Multi-GPU runs of bench.py are replicas: every rank counts its own copy of the workload and the
job time is the slowest rank's.  The aggregation is host logic, exercised here with two gloo
ranks on the CPU."""
import os
import socket
import sys

import pytest

torch = pytest.importorskip("torch")

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench
    seconds = [0.5, 2.0][rank]
    total = bench.max_over_ranks(seconds, world, torch.device("cpu"))
    out[rank] = (total, bench.replica_throughput(1e9, 4, total, world))
    dist.destroy_process_group()


def test_two_replicas_report_the_slowest_rank():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank_main, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(timeout=120)
            assert p.exitcode == 0
        res = dict(out)
    assert res[0] == res[1]
    total, value = res[0]
    assert total == 2.0
    assert value == pytest.approx(2 * 1e9 * 4 / 2.0)


def test_single_replica_is_unchanged():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(1.25, 1, None) == 1.25
    assert bench.replica_throughput(10.0, 3, 2.0, 1) == 15.0
