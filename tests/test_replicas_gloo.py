"""Multi-GPU is replicas only: each rank tracks its own trajectory, and the
only cross-rank step is the max of the elapsed times.  This exercises that
host-side logic with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import bench

    ms = [100.0 + 50.0 * rank, 300.0 - 100.0 * rank]
    red = bench.max_over_ranks(ms, "cpu", world)
    out[rank] = (red, bench.replica_throughput(10, world, red[0]))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_gloo():
    ctx = mp.get_context("spawn")
    with ctx.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [ctx.Process(target=_rank, args=(r, 2, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            red, thr = out[r]
            assert red == [150.0, 300.0]
            assert abs(thr - 20 / 0.150) < 1e-9


def test_single_rank_is_identity():
    import sys

    sys.path.insert(0, ROOT)
    import bench

    assert bench.max_over_ranks([1.0, 2.0], "cpu", 1) == [1.0, 2.0]
    assert bench.replica_throughput(5, 1, 1000.0) == 5.0
