"""The allocation-free entry point (pgb_react_boxes_noalloc) against the allocating one.

Callers such as PeleLM run on an AMReX arena that reserves most of the GPU up front; they need
a reactor call that allocates no device memory. This test drives that entry point through the
C ABI twice in a row (the fixed scratch array keeps the previous call's contents, so the second
call checks that the queue head and counters are cleared) and compares every output with
pgb_reactor_react_boxes on the same inputs, within the parity tolerances the other tests use
(T within 1e-6 relative, rhoY within atol + rtol |rhoY|): the 9-species mechanism through the
cell-per-thread kernel and the 21-species one through the cell-per-warp kernel. Free device
memory is read after a first call and again after the two compared calls: it must not change.
It is collected last so that a run stopping at the first failure has already run every other
test.
"""
import ctypes as C

import numpy as np
import pytest

from helpers import boxes_from_cells, gather, tol_ratio
from pelelm_gb300 import _lib
from pelelm_gb300.reactor import ReactorBase
from pelelm_gb300.workloads import CONFIGS, make_cells

SHAPES = [(8, 8, 8), (16, 4, 8), (5, 7, 3), (12, 6, 4)]
LOS = [(0, 0, 0), (8, -4, 2), (-3, 5, 100), (40, 40, 40)]


def _inputs(cfgname):
    cfg = CONFIGS[cfgname]
    n = sum(a * b * c for a, b, c in SHAPES)
    cs = make_cells(cfg, n, seed=17)
    rng = np.random.default_rng(2)
    cs.mask[:] = np.where(rng.uniform(size=n) < 0.1, -1, 1)
    return cfg, cs


def _noalloc(lib, cfg, boxes, precision):
    views = (_lib.BoxView * len(boxes))(*[b.view() for b in boxes])
    st = _lib.Stats()
    rc = lib.pgb_react_boxes_noalloc(cfg.mech.encode(), views, len(boxes), cfg.dt, cfg.rtol,
                                     cfg.atol, 5, 20000, int(precision == "fp64"), None, C.byref(st))
    assert rc == 0, _lib.last_error()
    return st


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("cfgname", ["lidryer_amr120", "drm19_2M"])
def test_noalloc_matches_allocating_entry(native_lib, cuda, cfgname, precision):
    torch = cuda
    cfg, cs = _inputs(cfgname)
    ns = cs.rY.shape[1]
    lib = _lib.lib()

    # reference: the allocating multi-box entry point with the same kernel family
    mapping = "thread" if ns <= 12 else "warp"
    boxes = boxes_from_cells(torch, cs, SHAPES, lo_list=LOS, ghost=1, with_mask=True)
    r = ReactorBase.create("ReactorCvode", cfg.mech,
                           f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.precision={precision} "
                           f"gb.mapping={mapping} gb.retry=0")
    r.init(2, 1)
    r.react_boxes(boxes, cfg.dt, 0.0)
    st_ref = r.stats()
    r.close()
    ref = gather(boxes, ns)

    # a first call loads the kernels and resolves the scratch array; from then on the device's
    # free memory must not move
    warm = boxes_from_cells(torch, cs, SHAPES, lo_list=LOS, ghost=1, with_mask=True)
    _noalloc(lib, cfg, warm, precision)
    inputs = [boxes_from_cells(torch, cs, SHAPES, lo_list=LOS, ghost=1, with_mask=True) for _ in range(2)]
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    stats = [_noalloc(lib, cfg, inputs[call], precision) for call in range(2)]
    torch.cuda.synchronize()
    free1 = torch.cuda.mem_get_info()[0]
    assert free1 == free0, f"device free memory moved by {free0 - free1} bytes"

    for call in range(2):
        st = stats[call]
        rY, T, rE, FC = gather(inputs[call], ns)
        assert st.nfail == 0 and st.ncell == st_ref["ncell"]
        assert st.nfe == st_ref["nfe"], f"call {call}: RHS counts differ"
        np.testing.assert_array_equal(FC, ref[3])
        assert np.max(np.abs(T - ref[1]) / ref[1]) <= 1e-6
        assert tol_ratio(rY, ref[0], cfg.rtol, cfg.atol).max() <= 1.0
        np.testing.assert_allclose(rE, ref[2], rtol=1e-14)


@pytest.mark.gpu
def test_noalloc_rejects_too_many_boxes(native_lib, cuda):
    cfg, _ = _inputs("lidryer_amr120")
    n = 1025  # one more than PGB_NOALLOC_MAX_BOXES
    views = (_lib.BoxView * n)()
    rc = _lib.lib().pgb_react_boxes_noalloc(cfg.mech.encode(), views, n, cfg.dt, cfg.rtol, cfg.atol,
                                            5, 20000, 1, None, None)
    assert rc == -1
    assert "exceed" in _lib.last_error()


@pytest.mark.gpu
def test_noalloc_captures_and_replays(native_lib, cuda):
    """A call captured into a CUDA graph replays to the same outputs as a direct call on the
    same inputs (the box table travels in kernel parameters, so nothing the graph refers to
    dies with the call); asking for stats while the stream is capturing is refused before any
    work is recorded, and leaves the capture usable."""
    torch = cuda
    cfg, cs = _inputs("drm19_2M")
    ns = cs.rY.shape[1]
    lib = _lib.lib()
    _noalloc(lib, cfg, boxes_from_cells(torch, cs, SHAPES, lo_list=LOS, ghost=1, with_mask=True), "mixed")
    direct = boxes_from_cells(torch, cs, SHAPES, lo_list=LOS, ghost=1, with_mask=True)
    _noalloc(lib, cfg, direct, "mixed")
    ref = gather(direct, ns)

    captured = boxes_from_cells(torch, cs, SHAPES, lo_list=LOS, ghost=1, with_mask=True)
    views = (_lib.BoxView * len(captured))(*[b.view() for b in captured])
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, capture_error_mode="thread_local"):
        sptr = torch.cuda.current_stream().cuda_stream
        st = _lib.Stats()
        rc = lib.pgb_react_boxes_noalloc(cfg.mech.encode(), views, len(captured), cfg.dt, cfg.rtol,
                                         cfg.atol, 5, 20000, 0, C.c_void_p(sptr), C.byref(st))
        assert rc == -1 and "capture" in _lib.last_error()
        rc = lib.pgb_react_boxes_noalloc(cfg.mech.encode(), views, len(captured), cfg.dt, cfg.rtol,
                                         cfg.atol, 5, 20000, 0, C.c_void_p(sptr), None)
        assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    before = gather(captured, ns)
    np.testing.assert_array_equal(before[3], 0.0)  # capture records, it does not run
    g.replay()
    torch.cuda.synchronize()
    out = gather(captured, ns)
    for a, b in zip(out, ref):
        np.testing.assert_array_equal(a, b)
