"""The N>1 bench path on CPU: two gloo ranks run replicas; the timed region ends with a
max-over-ranks of the per-rank times, and the job rate counts every rank's units."""
import os
import socket

import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, ws, port, q):
    import sys
    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    t_local = 1.0 + rank  # rank 1 is the slow one
    out = (bench.reduce_max(t_local, ws), bench.job_rate(1000.0, ws, t_local))
    dist.barrier()
    dist.destroy_process_group()
    q.put((rank, out))


@pytest.mark.timeout(120)
def test_two_rank_replica_timing():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
        assert p.exitcode == 0
    for r in (0, 1):
        t_max, rate = res[r]
        assert t_max == 2.0                 # the slowest rank's time, on every rank
        assert rate == pytest.approx(1000.0 * 2 / 2.0)


def test_single_rank_is_identity():
    import sys
    sys.path.insert(0, ROOT)
    import bench
    assert bench.reduce_max(3.5, 1) == 3.5
    assert bench.job_rate(10.0, 1, 2.0) == 5.0
