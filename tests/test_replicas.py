"""Multi-GPU is replicas only (independent swarms per rank, no data-path
collective).  The bench's rank plumbing, barrier and max-over-ranks timing,
runs here as two gloo ranks on CPU."""
import os
import socket
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, ws, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(ws),
                      LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import torch.distributed as dist
    dist.init_process_group("gloo", rank=rank, world_size=ws)
    import bench
    # each rank "measures" a different time; every rank must see the maximum
    got = bench._barrier_max(1.0 + rank, ws)
    bench._barrier(ws)
    q.put((rank, got, bench._dist()))
    dist.destroy_process_group()


@pytest.mark.timeout(120)
def test_two_rank_max_over_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=100) for _ in procs)
    for p in procs:
        p.join(timeout=30)
    assert [r[1] for r in res] == [2.0, 2.0]
    assert [r[2] for r in res] == [(2, 0), (2, 1)]
