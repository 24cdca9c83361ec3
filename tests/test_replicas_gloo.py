"""Multi-GPU mode is replicas only: each rank plans its own query and the
job's throughput is all ranks' units over the slowest rank's time.  The
aggregation runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, q):
    import sys
    import torch.distributed as dist
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    units, times = bench.aggregate(dist, 1000 + 10 * rank, [5.0 + rank, 7.0 - rank])
    q.put((rank, units, times))
    dist.destroy_process_group()


def test_replica_aggregation_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, units, times in out:
        assert units == pytest.approx(2010.0)
        assert times == pytest.approx([6.0, 7.0])


def test_single_process_passthrough():
    import bench
    assert bench.aggregate(None, 5, [1.0, 2.0]) == (5, [1.0, 2.0])
