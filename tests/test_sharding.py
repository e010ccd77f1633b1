"""Host-side partition of a box list across ranks (pgb_chop_boxes / pgb_partition_boxes through
the C ABI; no GPU): pieces tile their parent boxes, the greedy bound holds, edge cases."""
import numpy as np
import pytest

from pelelm_gb300.sharding import box_cells, chop_boxes, partition_boxes


def test_chop_tiles_the_parents_and_respects_min_side(native_lib):
    boxes = [((0, 0, 0), (63, 63, 63)), ((-8, 4, 100), (7, 11, 131)), ((5, 5, 5), (12, 12, 12))]
    pieces, parent = chop_boxes(boxes, 16, 64)
    assert 8 < len(pieces) <= 64
    for b, box in enumerate(boxes):
        mine = [p for p, q in zip(pieces, parent) if q == b]
        assert sum(box_cells(p) for p in mine) == box_cells(box)
        cover = set()
        for lo, hi in mine:
            assert all(lo[d] >= box[0][d] and hi[d] <= box[1][d] for d in range(3))
            cells = {(i, j, k) for i in range(lo[0], hi[0] + 1) for j in range(lo[1], hi[1] + 1)
                     for k in range(lo[2], hi[2] + 1)} if box_cells((lo, hi)) <= 5000 else None
            if cells is not None:
                assert not (cover & cells)
                cover |= cells
    # a side is split only when both halves keep min_side cells; the 8^3 box stays whole
    assert [p for p, q in zip(pieces, parent) if q == 2] == [boxes[2]]
    for (lo, hi), q in zip(pieces, parent):
        if q != 2:
            assert min(hi[d] - lo[d] + 1 for d in range(3)) >= 8


def test_chop_stops_at_target_and_rejects_bad_input(native_lib):
    boxes = [((0, 0, 0), (31, 31, 31))]
    pieces, parent = chop_boxes(boxes, 4, 5)
    assert len(pieces) == 5 and set(parent) == {0}
    pieces, _ = chop_boxes(boxes, 64, 100)  # nothing can be split
    assert pieces == boxes
    with pytest.raises(RuntimeError, match="empty"):
        chop_boxes([((0, 0, 0), (-1, 3, 3))], 4, 8)


@pytest.mark.parametrize("nranks", [1, 2, 3, 8, 40])
def test_partition_is_complete_and_within_the_greedy_bound(native_lib, nranks):
    rng = np.random.default_rng(nranks)
    w = np.concatenate([rng.uniform(0, 1, 30), rng.uniform(5, 50, 5), [0.0, 0.0]])
    ranks, load = partition_boxes(w, nranks)
    assert ranks.shape == w.shape and ranks.min() >= 0 and ranks.max() < nranks
    np.testing.assert_allclose([w[ranks == r].sum() for r in range(nranks)], load, rtol=0, atol=1e-12)
    assert load.max() <= load.mean() + w.max() + 1e-12
    # never worse than the trivial lower bounds by more than the greedy factor 4/3
    assert load.max() <= 4.0 / 3.0 * max(w.sum() / nranks, w.max()) + 1e-12
    again, _ = partition_boxes(w, nranks)
    assert np.array_equal(ranks, again), "deterministic"


def test_partition_edge_cases(native_lib):
    ranks, load = partition_boxes([], 4)
    assert ranks.size == 0 and np.all(load == 0)
    ranks, load = partition_boxes([3.0, 3.0, 2.0, 2.0, 2.0], 2)
    assert sorted(load) == [6.0, 6.0]
    with pytest.raises(RuntimeError, match="negative"):
        partition_boxes([1.0, -1.0], 2)
    with pytest.raises(RuntimeError, match="nranks"):
        partition_boxes([1.0], 0)
