"""GPU parity of the warp-per-cell BDF kernel (gb.mapping=warp; the only mapping compiled for
the GRI-shaped mechanism, 53 species / 325 reactions) and of the lane-group kernel
(gb.mapping=group, 4 or 8 lanes per cell; the drm19-shaped default) against the CPU oracle,
through the C ABI.

The warp kernel sums production rates, norms and the energy closure in a different order than
the oracle (lanes, shuffles), so a cell can take a different step sequence; FP64 mode is held
to the plain method's tolerances (T within 1e-6 relative, rhoY within atol + rtol |rhoY|) on
at least 99% of the cells and, like mixed precision, judged on all cells by its error against a
tight oracle (rtol 1e-11), which must be no worse than the FP64 oracle's own error at the same
rtol/atol.
"""
import json
import os

import numpy as np
import pytest

from helpers import boxes_from_cells, gather, outliers_within_global_error, tol_ratio
from pelelm_gb300.reactor import ReactorBase
from pelelm_gb300.workloads import CONFIGS, make_cells, mech_path

OUT = os.environ.get("PGB_TEST_OUT", "test_reports")


def _report(name, d):
    try:
        os.makedirs(OUT, exist_ok=True)
        with open(os.path.join(OUT, "parity_report.jsonl"), "a") as f:
            f.write(json.dumps({"test": name, **d}) + "\n")
    except OSError:
        pass


def _run(torch, cfg, cs, sides, opts, **kw):
    boxes = boxes_from_cells(torch, cs, sides, **kw)
    r = ReactorBase.create("ReactorCvode", cfg.mech, f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} {opts}")
    r.init(2, 1)
    r.react_boxes(boxes, cfg.dt, 0.0)
    torch.cuda.synchronize()
    st = r.stats()
    r.close()
    return gather(boxes, cs.rY.shape[1]), st


CASES = [("lidryer_amr120", 2048, [8, 8, 8, 8], "gb.mapping=warp"),
         ("drm19_2M", 1024, [8, 8], "gb.mapping=warp"),
         ("drm19_2M", 8192, [16, 16], "gb.mapping=group gb.group=8"),
         ("drm19_2M", 4096, [16], "gb.mapping=group gb.group=4"),
         ("gri_1M", 2048, [(16, 16, 8)], "")]


def _errs(tight, rY, T):
    Yt = tight[0] / tight[0].sum(1, keepdims=True)
    Y = rY / rY.sum(1, keepdims=True)
    dT = np.abs(T - tight[1])
    dY = np.abs(Y - Yt).max(1)
    return dT.max(), np.percentile(dT, 99), dY.max(), np.percentile(dY, 99)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("cfgname,n,sides,opts", CASES)
def test_warp_kernel_against_oracle(native_lib, oracle_mod, cuda, cfgname, n, sides, opts, precision):
    cfg = CONFIGS[cfgname]
    cs = make_cells(cfg, n, seed=21)
    (rYg, Tg, rEg, FCg), st = _run(cuda, cfg, cs, sides, f"{opts} gb.precision={precision}")
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    rYo, To, rEo, FCo, nf = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, cfg.rtol, cfg.atol)
    tight = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, 1e-11, 1e-16, max_steps=200000)
    # A few GRI-shaped cells per 10^4 fail in any FP64 BDF (Newton convergence failures; the
    # oracle fails the same ones): cells the oracle fails may fail here too, no other cell may,
    # and the comparisons run over the cells both sides integrate.
    ok = (FCo > 0) & (FCg > 0)
    assert np.all(FCg[FCo > 0] > 0), "a cell the oracle integrates failed on the GPU"
    assert nf <= max(2, n // 1000)
    relT = np.abs(Tg - To)[ok] / To[ok]
    ratio = tol_ratio(rYg[ok], rYo[ok], cfg.rtol, cfg.atol).max(1)
    within = (relT <= 1e-6) & (ratio <= 1.0)
    tok = tight[3] > 0
    sel = ok & tok
    tsel = tuple(x[sel] if getattr(x, "ndim", 0) else x for x in tight)
    eg, eo = _errs(tsel, rYg[sel], Tg[sel]), _errs(tsel, rYo[sel], To[sel])
    _report(f"warp[{cfgname},{precision}]", {
        "cells": int(n), "frac_within_plain_tol": float(within.mean()), "max_relT": float(relT.max()),
        "max_ratio": float(ratio.max()), "frac_same_nfe": float(np.mean(FCg[ok] == FCo[ok])),
        "nfe_gpu": float(FCg[ok].mean()), "nfe_orc": float(FCo[ok].mean()), "nfail": int(st["nfail"]),
        "nfail_oracle": int(nf),
        "err_vs_tight_gpu": [float(x) for x in eg], "err_vs_tight_oracle": [float(x) for x in eo]})
    np.testing.assert_allclose(rEg[ok], rEo[ok], rtol=1e-14, atol=1e-14 * np.abs(rEo).max())
    if precision == "fp64":
        assert within.mean() >= 0.99, within.mean()
        # every cell outside the plain tolerances is held, cell by cell, to the oracle's own
        # global error on that cell against the tight oracle
        out = np.nonzero(ok)[0][~within]
        outliers_within_global_error(om, cs, out, (rYg[out], Tg[out]), (rYo[out], To[out]), cfg.dt, cfg.rtol)
    Tmax = float(np.max(tight[1]))
    bounds = ((2.0, 50 * cfg.rtol * Tmax), (1.25, 1e-3), (2.0, 50 * cfg.rtol), (1.25, 1e-8))
    for a, b, (fac, slack) in zip(eg, eo, bounds):
        assert a <= fac * b + slack, (eg, eo)


@pytest.mark.gpu
def test_warp_kernel_boxes_ghosts_mask_graph(native_lib, oracle_mod, cuda):
    """Uneven boxes with offsets, ghost cells and a mask in one launch, also from a CUDA graph."""
    torch = cuda
    cfg = CONFIGS["lidryer_amr120"]
    shapes = [(8, 8, 8), (16, 4, 8), (5, 7, 3), (12, 6, 4)]
    n = sum(a * b * c for a, b, c in shapes)
    cs = make_cells(cfg, n, seed=3)
    rng = np.random.default_rng(5)
    cs.mask[:] = np.where(rng.uniform(size=n) < 0.1, -1, 1)
    los = [(0, 0, 0), (8, -4, 2), (-3, 5, 100), (40, 40, 40)]
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    rYo, To, rEo, FCo, nf = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, cfg.rtol, cfg.atol)
    stream = torch.cuda.Stream()
    boxes = boxes_from_cells(torch, cs, shapes, lo_list=los, ghost=2, with_mask=True)
    r = ReactorBase.create("ReactorCvode", cfg.mech, f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.graph=1 "
                           "gb.precision=fp64 gb.mapping=warp")
    r.init(2, 1)
    for rep in range(2):
        if rep:
            boxes = boxes_from_cells(torch, cs, shapes, lo_list=los, ghost=2, with_mask=True)
        with torch.cuda.stream(stream):
            r.react_boxes(boxes, cfg.dt, 0.0, stream=stream)
        stream.synchronize()
        rYg, Tg, rEg, FCg = gather(boxes, cs.rY.shape[1])
        covered = cs.mask < 0
        assert np.all(FCg[covered] == 0) and np.all(FCg[~covered] > 0)
        np.testing.assert_array_equal(Tg[covered], cs.T[covered])
        np.testing.assert_array_equal(rYg[covered], cs.rY[covered])
        relT = (np.abs(Tg - To) / To)[~covered]
        assert np.mean(relT <= 1e-6) >= 0.99
    r.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mapping", ["warp", "group"])
def test_warp_kernel_is_deterministic_and_serves_the_surrogate_fallback(native_lib, cuda, mapping):
    """Two runs give identical bits (no atomics in the arithmetic); the surrogate's fallback
    cells through the warp (or lane-group) kernel equal the plain run bit for bit."""
    torch = cuda
    cfg = CONFIGS["drm19_2M"]
    cs = make_cells(cfg, 4096, seed=31)
    base = f"gb.mapping={mapping} gb.precision=mixed"
    (a, _), (b, _) = (_run(torch, cfg, cs, [16], base) for _ in range(2))
    for x, y in zip(a, b):
        assert np.array_equal(x, y)
    surr = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "pelelm_gb300", "data",
                        "drm19_syn.pgbs")
    with open(surr + ".levels.json") as f:
        lv = json.load(f)["levels"][-1]
    sg = " ".join(f"gb.sg.{k}={lv[k]!r}" for k in ("mis", "cons", "disT", "disY", "neg", "tol_T", "tol_Y"))
    (g, _) = _run(torch, cfg, cs, [16], f"{base} gb.surrogate={surr} {sg}")
    fb = g[3] != 0.0
    assert fb.any() and (~fb).any()
    assert np.array_equal(g[0][fb], a[0][fb]) and np.array_equal(g[1][fb], a[1][fb])


@pytest.mark.gpu
def test_gri_thread_mapping_and_pointwise_rates_are_refused(native_lib, cuda):
    with pytest.raises(RuntimeError, match="cell-per-thread"):
        ReactorBase.create("ReactorCvode", "gri_syn", "gb.mapping=thread").init(2, 1)
    with pytest.raises(RuntimeError, match="surrogate"):
        ReactorBase.create("ReactorCvode", "gri_syn", "gb.surrogate=x.pgbs").init(2, 1)


@pytest.mark.gpu
@pytest.mark.parametrize("cfgname", ["drm19_2M", "lidryer_amr120"])
def test_autotuner_picks_a_compiled_mapping_and_leaves_inputs_alone(native_lib, cuda, cfgname):
    """gb.autotune=1 times every compiled mapping on a sample of the first call's cells and
    keeps the fastest; the advance then equals, bit for bit, one made with that mapping given
    explicitly (so the tuning only read the caller's arrays)."""
    torch = cuda
    cfg = CONFIGS[cfgname]
    cs = make_cells(cfg, 4 * 16 ** 3, seed=8)
    (a, _) = _run(torch, cfg, cs, [16] * 4, "gb.precision=mixed gb.autotune=1")
    r = ReactorBase.create("ReactorCvode", cfg.mech, f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.autotune=1")
    r.init(2, 1)
    r.react_boxes(boxes_from_cells(torch, cs, [16] * 4), cfg.dt, 0.0)
    torch.cuda.synchronize()
    rep = r.tuning()
    r.close()
    _report(f"autotune[{cfgname}]", {"report": rep})
    assert "->" in rep and "thread" in rep and "warp/" in rep
    if cfgname.startswith("drm19"):
        assert "group/8" in rep and "group/4" in rep
    picked = rep.split("->")[-1].strip()
    kind, _, size = picked.partition("/")
    explicit = {"thread": "gb.mapping=thread", "warp": f"gb.mapping=warp gb.wpb={size}",
                "group": f"gb.mapping=group gb.group={size}"}[kind]
    (b, _) = _run(torch, cfg, cs, [16] * 4, "gb.precision=mixed " + explicit)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def _run_graph_twice(torch, cfg, cs, sides, opts):
    """Two advances of fresh copies of the same cells through one cached CUDA graph."""
    stream = torch.cuda.Stream()
    r = ReactorBase.create("ReactorCvode", cfg.mech, f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.graph=1 {opts}")
    r.init(2, 1)
    outs = []
    for _ in range(2):
        boxes = boxes_from_cells(torch, cs, sides)
        with torch.cuda.stream(stream):
            r.react_boxes(boxes, cfg.dt, 0.0, stream=stream)
        stream.synchronize()
        outs.append((gather(boxes, cs.rY.shape[1]), r.stats()))
    r.close()
    return outs


@pytest.mark.gpu
@pytest.mark.parametrize("cfgname,mapping", [("lidryer_amr120", "thread"), ("drm19_2M", "warp"),
                                             ("drm19_2M", "group")])
def test_mixed_precision_retries_failed_cells_in_fp64(native_lib, cuda, cfgname, mapping):
    """gb.retry (on by default in mixed precision): a cell the mixed-precision pass fails is
    integrated again, from its untouched inputs, by the FP64 kernel in the same call (and the
    same CUDA graph). A step limit below the cells' step counts makes failures certain: each
    retried cell then equals the plain FP64 run bit for bit, every other cell the mixed run
    without retry, and the counters split into nretry (handed over) and nfail (failed in FP64)."""
    torch = cuda
    cfg = CONFIGS[cfgname]
    cs = make_cells(cfg, 4096, seed=12)
    lim = f"gb.mapping={mapping} ode.max_steps=40"
    (a, sa) = _run(torch, cfg, cs, [16], f"{lim} gb.precision=mixed gb.retry=0")
    (d, sd) = _run(torch, cfg, cs, [16], f"{lim} gb.precision=fp64")
    failed = a[3] < 0
    assert 0 < failed.sum() < failed.size and sa["nretry"] == 0 and sa["nfail"] == failed.sum()
    for (g, sg) in _run_graph_twice(torch, cfg, cs, [16], f"{lim} gb.precision=mixed"):
        for x, y, z in zip(g, a, d):
            assert np.array_equal(x[~failed], y[~failed])
            assert np.array_equal(x[failed], z[failed])
        assert sg["nretry"] == failed.sum()
        assert sg["nfail"] == (d[3][failed] < 0).sum()
    _report(f"retry[{cfgname}]", {"cells": int(failed.size), "mixed_failed": int(failed.sum()),
                                  "failed_after_fp64_retry": int(sg["nfail"]), "fp64_alone_failed": int(sd["nfail"])})


@pytest.mark.gpu
def test_gri_mixed_with_retry_fails_no_more_cells_than_fp64(native_lib, cuda):
    """On the GRI-shaped workload a few cells per 10^4 fail the FP32-Newton mixed pass (and a
    similar number fail in FP64, as they do in the oracle). The sample holds such cells; with
    the retry the mixed advance fails only cells that FP64 fails as well."""
    torch = cuda
    cfg = CONFIGS["gri_1M"]
    full = make_cells(cfg, 65536, seed=0)
    known = [480, 728, 7950, 9836, 12643, 13753, 15664, 15833, 18082, 19744, 25373, 29068, 30942,
             31718, 33513, 34007, 35261, 40001, 40191, 42264, 42733, 43442, 47339, 50746, 61635, 65528]
    rng = np.random.default_rng(9)
    others = rng.choice(np.setdiff1d(np.arange(65536), known), 256 - len(known), replace=False)
    sel = np.sort(np.concatenate([known, others]))
    cs = type(full)(**{k: (v[sel] if isinstance(v, np.ndarray) and v.shape[:1] == (65536,) else v)
                       for k, v in full.__dict__.items()})
    shape = [(16, 16, 1)]
    (a, sa) = _run(torch, cfg, cs, shape, "gb.precision=mixed gb.retry=0")
    (d, sd) = _run(torch, cfg, cs, shape, "gb.precision=fp64")
    (g, sg) = _run(torch, cfg, cs, shape, "gb.precision=mixed")
    failed = a[3] < 0
    for x, y, z in zip(g, a, d):
        assert np.array_equal(x[~failed], y[~failed]) and np.array_equal(x[failed], z[failed])
    assert sg["nretry"] == failed.sum() and sg["nfail"] == (d[3][failed] < 0).sum()
    assert sg["nfail"] <= min(sa["nfail"], sd["nfail"])
    _report("retry[gri_1M]", {"cells": 256, "mixed_failed": int(sa["nfail"]), "fp64_failed": int(sd["nfail"]),
                              "mixed_with_retry_failed": int(sg["nfail"])})
