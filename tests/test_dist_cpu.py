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


def _shard_worker(rank, world, port, q):
    """One rank of a sharded chemistry advance: chop the global box list, partition it by cell
    count, advance the own shard (the CPU oracle stands in for the GPU kernels), exchange the
    per-box FC sums, partition again by FC weight and advance the new shard."""
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    import numpy as np
    import oracle as O
    from pelelm_gb300.sharding import box_cells, chop_boxes, fc_weights, partition_boxes
    from pelelm_gb300.workloads import CONFIGS, make_cells, mech_path
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = CONFIGS["lidryer_amr120"]
    sides = [16, 8, 8, 4, 12, 8]
    boxes = [((0, 0, 32 * b), (s - 1, s - 1, 32 * b + s - 1)) for b, s in enumerate(sides)]
    pieces, parent = chop_boxes(boxes, 4, 4 * world)
    ncell = sum(box_cells(p) for p in pieces)
    cs = make_cells(cfg, ncell, seed=3)          # cell state in piece order
    off = np.cumsum([0] + [box_cells(p) for p in pieces])
    om = O.OracleMech(mech_path(cfg.mech))
    results = []
    weights = np.array([box_cells(p) for p in pieces], dtype=np.float64)
    for rnd in range(2):
        ranks, load = partition_boxes(weights, world)
        mine = [b for b in range(len(pieces)) if ranks[b] == rank]
        cells = np.concatenate([np.arange(off[b], off[b + 1]) for b in mine]) if mine else np.zeros(0, int)
        out = om.react(cs.rY[cells], cs.rYsrc[cells], cs.T[cells], cs.rE[cells], cs.rEsrc[cells], cs.mask[cells],
                       cfg.dt, cfg.rtol, cfg.atol, nthreads=1)
        fc_mine = {b: out[3][np.searchsorted(cells, np.arange(off[b], off[b + 1]))] for b in mine}
        gathered = [None] * world
        dist.all_gather_object(gathered, (rank, ranks.tolist(), mine, cells.tolist(),
                                          [x.tolist() if hasattr(x, "tolist") else x for x in out[:4]],
                                          {b: float(fc_weights([fc_mine[b]])[0]) for b in mine}))
        results.append((load.tolist(), weights.tolist(), gathered))
        w = {}
        for g in gathered:
            w.update(g[5])
        weights = np.array([w[b] for b in range(len(pieces))])
    if rank == 0:
        full = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, cfg.rtol, cfg.atol, nthreads=1)
        q.put((len(pieces), parent.tolist(), [p for p in pieces], results,
               [x.tolist() if hasattr(x, "tolist") else x for x in full[:4]]))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_sharded_advance_is_complete_balanced_and_equals_one_rank():
    """World size 2 on gloo: both ranks compute the same partition; the shards are disjoint and
    cover every box; the largest load stays within the mean load plus the heaviest box (the
    bound of the greedy partition) in both rounds (cell counts, then the FC weights of the first
    advance); and the shards' results put together equal the one-rank advance bit for bit."""
    import numpy as np
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_shard_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    npieces, parent, pieces, results, full = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert npieces >= 8 and sorted(set(parent)) == list(range(6))
    for load, weights, gathered in results:
        assert gathered[0][1] == gathered[1][1], "ranks computed different partitions"
        boxes_seen = sorted(b for g in gathered for b in g[2])
        assert boxes_seen == list(range(npieces)), "shards must be disjoint and complete"
        w = np.array(weights)
        assert max(load) <= np.mean(load) + w.max() + 1e-9
        assert abs(sum(load) - w.sum()) <= 1e-9 * w.sum()
        cells = np.concatenate([np.array(g[3], dtype=int) for g in gathered])
        assert np.array_equal(np.sort(cells), np.arange(len(full[1])))
        for k in range(4):
            merged = np.empty_like(np.array(full[k]))
            for g in gathered:
                merged[np.array(g[3], dtype=int)] = np.array(g[4][k])
            assert np.array_equal(merged, np.array(full[k])), f"output {k} differs from the one-rank advance"
