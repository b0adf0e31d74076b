"""bench.py --gpus N runs N independent replicas (the path is not sharded:
one GPU per copy, no data-path collective).  Its only collectives are the
barrier around the timed region and the max over ranks of the elapsed time,
from which the whole-job throughput is formed.  Checked here on two gloo
ranks on the CPU (127.0.0.1 rendezvous)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, out):
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    try:
        import bench
        local = 1.0 + rank            # rank 1 is the slower replica
        bench.barrier(ws)
        value, elapsed = bench.replica_throughput(1000.0, local, ws)
        out.put((rank, value, elapsed))
    finally:
        dist.destroy_process_group()


def test_replica_throughput_is_max_over_two_gloo_ranks():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    for rank, value, elapsed in res:
        assert elapsed == pytest.approx(2.0)          # the slowest rank's time on every rank
        assert value == pytest.approx(2 * 1000.0 / 2.0)   # all units of both replicas over that time


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.replica_throughput(500.0, 2.0, 1) == (250.0, 2.0)
