"""bench.py's multi-rank aggregation on CPU: two gloo ranks, barrier, the
max over ranks of the timed region and the sum of the samples processed
(replicas: each rank runs its own stream)."""
import os
import socket
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, port, q):
    sys.path.insert(0, ROOT)
    os.environ.update(WORLD_SIZE="2", RANK=str(rank), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    import bench
    ws, r = bench.dist_init("gloo")
    bench.dist_barrier()
    t = bench.dist_max(1.5 + rank)          # rank 1 is the slow one
    n = bench.dist_sum(100 * (rank + 1))
    q.put((r, ws, t, n))
    import torch.distributed as dist
    dist.destroy_process_group()


def test_two_rank_aggregation():
    mp = pytest.importorskip("torch.multiprocessing")
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    ps = [ctx.Process(target=_worker, args=(r, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = sorted(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
    assert [r[0] for r in res] == [0, 1]
    for r, ws, t, n in res:
        assert ws == 2 and t == 2.5 and n == 300
