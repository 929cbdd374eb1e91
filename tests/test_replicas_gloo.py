"""World-size-2 test of the replicas path of bench.py on CPU (gloo): the
slowest rank's time is taken and the whole-job value counts every rank."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, q):
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    t = bench.max_over_ranks(1.0 + rank, world)
    q.put((rank, t, bench.replica_value(10, world, t)))
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks():
    mp = pytest.importorskip("torch.multiprocessing")
    import socket
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, t, v in out:
        assert t == 2.0
        assert v == pytest.approx(2 * 10 / 2.0)


def test_single_rank_is_local():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.replica_value(5, 1, 2.0) == 2.5
