"""Sharding of one chemistry box list across ranks (one rank per GPU), weighted by cost.

Host-side mirror of the partition calls of the native library (include/pelelm_gb300.h,
``pgb_chop_boxes`` / ``pgb_partition_boxes``), the analogue of PeleLM's chemistry load balance:
grids chopped until each rank has enough boxes (Source/PeleLM.cpp:5699-5723), then a knapsack
over each box's FuncCount sum of the previous advance (getFuncCountDM,
Source/PeleLM.cpp:5530-5623). Every cell is an independent ODE, so a rank advances its shard
with no collective on the data path; only the per-box weights are exchanged between advances.
"""
from __future__ import annotations

import ctypes as C
from typing import List, Sequence, Tuple

import numpy as np

from . import _lib

Box = Tuple[Tuple[int, int, int], Tuple[int, int, int]]


def chop_boxes(boxes: Sequence[Box], min_side: int, target: int) -> Tuple[List[Box], np.ndarray]:
    """Pieces of the boxes (largest halved across its longest side first, no side below
    min_side) until there are `target` of them or none can be split; returns the pieces and the
    index of each piece's parent box."""
    n = len(boxes)
    cap = max(n, int(target))
    src = (_lib.Box * max(n, 1))()
    for b, (lo, hi) in enumerate(boxes):
        for d in range(3):
            src[b].lo[d], src[b].hi[d] = int(lo[d]), int(hi[d])
    out = (_lib.Box * max(cap, 1))()
    parent = (C.c_int * max(cap, 1))()
    m = _lib.check(_lib.lib().pgb_chop_boxes(src, n, int(min_side), int(target), out, parent, cap), "chop_boxes")
    pieces = [(tuple(out[i].lo), tuple(out[i].hi)) for i in range(m)]
    return pieces, np.array(parent[:m], dtype=np.int64)


def partition_boxes(weights: Sequence[float], nranks: int) -> Tuple[np.ndarray, np.ndarray]:
    """rank of every box and the load of every rank (weights: FC sums or cell counts)."""
    w = np.ascontiguousarray(weights, dtype=np.float64)
    n = w.size
    ranks = np.zeros(max(n, 1), dtype=np.int32)
    load = np.zeros(nranks, dtype=np.float64)
    _lib.check(_lib.lib().pgb_partition_boxes(w.ctypes.data, n, int(nranks), ranks.ctypes.data,
                                             load.ctypes.data), "partition_boxes")
    return ranks[:n], load


def box_cells(box: Box) -> int:
    lo, hi = box
    return int(np.prod([hi[d] - lo[d] + 1 for d in range(3)]))


def fc_weights(fc_per_box: Sequence) -> np.ndarray:
    """Per-box work of the last advance from each box's FC array (tensor or numpy): the sum of
    the RHS-evaluation counts of its cells (failed cells, FC < 0, and covered cells count 0)."""
    out = []
    for fc in fc_per_box:
        a = fc.double().clamp(min=0).sum().item() if hasattr(fc, "clamp") else float(np.clip(fc, 0, None).sum())
        out.append(a)
    return np.array(out, dtype=np.float64)
