"""Multi-rank plumbing of bench.py on CPU (gloo, world size 2): each rank advances its own shard
of cells (weak scaling, no collective on the data path); only the timing max and the cell
totals are reduced."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402


def _worker(rank, world, port, q):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import bench

    class A:
        impl = "reference"
    ws, r, local, pg = bench.dist_setup(A)
    t = 1.0 + r           # per-rank time
    cells = 100.0 * (r + 1)
    out = (ws, r, bench.allmax(pg, t), bench.allsum(pg, cells))
    q.put(out)
    pg.destroy_process_group()


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def test_two_rank_reductions():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
    assert [r[1] for r in res] == [0, 1]
    for ws, r, tmax, csum in res:
        assert ws == 2 and tmax == 2.0 and csum == 300.0
