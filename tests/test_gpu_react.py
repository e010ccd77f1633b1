"""GPU parity: the GB300 reactor (through the C ABI) against the CPU oracle on the same seeded
inputs.

Tolerances are the ones the benchmark definition states for the plain method at
ode.rtol / ode.atol: temperature within 1e-6 relative, every rhoY within atol + rtol*|rhoY|.
Both sides run the same CVODE-class algorithm, so these hold cell by cell; rho h must match to
round-off (it is rho h0 + F_h dt on both sides).
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


def _run_both(torch, oracle_mod, cfg, n, seed, precision, sides):
    cs = make_cells(cfg, n, seed=seed)
    boxes = boxes_from_cells(torch, cs, sides)
    r = ReactorBase.create("ReactorCvode", cfg.mech,
                           f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.precision={precision}")
    r.init(2, 1)
    nfail = 0
    for b in boxes:
        nfail += r.react(b.box, b.rY, b.rY_src, b.T, b.rEner, b.rEner_src, b.FC, b.mask, cfg.dt, 0.0)
    torch.cuda.synchronize()
    g = gather(boxes, cs.rY.shape[1])
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    o = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, cfg.rtol, cfg.atol)
    r.close()
    return cs, g, o, nfail


@pytest.mark.gpu
@pytest.mark.parametrize("cfgname,n,sides", [("lidryer_32cube", 32768, [32]),
                                             ("lidryer_amr120", 2048, [8, 8, 8, 8]),
                                             ("drm19_2M", 16384, [16, 16, 16, 16])])
def test_react_fp64_matches_oracle(native_lib, oracle_mod, cuda, cfgname, n, sides):
    """Plain method (FP64 Jacobian and LU) against the oracle at the same rtol/atol."""
    precision = "fp64"
    torch = cuda
    cfg = CONFIGS[cfgname]
    cs, g, o, nfail = _run_both(torch, oracle_mod, cfg, n, 7, precision, sides)
    rYg, Tg, rEg, FCg = g
    rYo, To, rEo, FCo, nfail_o = o
    relT = np.abs(Tg - To) / To
    ratio = tol_ratio(rYg, rYo, cfg.rtol, cfg.atol)
    same_nfe = float(np.mean(FCg == FCo))
    _report(f"react[{cfgname},{precision}]", {
        "max_relT": float(relT.max()), "p99_relT": float(np.percentile(relT, 99)),
        "max_ratio": float(ratio.max()), "p99_ratio": float(np.percentile(ratio, 99)),
        "frac_same_nfe": same_nfe, "nfe_gpu": float(FCg.mean()), "nfe_orc": float(FCo.mean()),
        "nfail": int(nfail), "nfail_oracle": int(nfail_o), "cells": int(n),
        "frac_within_plain_tol": float(np.mean((relT <= 1e-6) & (ratio.max(1) <= 1.0)))})
    assert nfail == 0 and nfail_o == 0
    assert np.all(FCg > 0)
    # rho h crosses zero for fuel-rich CH4/air, so judge it on the scale of the field
    np.testing.assert_allclose(rEg, rEo, rtol=1e-14, atol=1e-14 * np.abs(rEo).max())
    # cell by cell within the plain tolerances; the rare cell that took another step sequence
    # (rate code and oracle differ in the last bit) is held to the oracle's own global error
    within = (relT <= 1e-6) & (tol_ratio(rYg, rYo, cfg.rtol, cfg.atol).max(1) <= 1.0)
    assert within.mean() >= 0.999, f"{within.mean():.5f} of cells within the plain tolerances"
    out = np.nonzero(~within)[0]
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    outliers_within_global_error(om, cs, out, (rYg[out], Tg[out]), (rYo[out], To[out]), cfg.dt, cfg.rtol)
    # same algorithm in the same precision: step/RHS counts agree on almost every cell
    assert same_nfe >= 0.9


@pytest.mark.gpu
@pytest.mark.parametrize("cfgname,n,sides", [("lidryer_32cube", 32768, [32]),
                                             ("lidryer_amr120", 2048, [8, 8, 8, 8]),
                                             ("drm19_2M", 16384, [16, 16, 16, 16])])
def test_react_mixed_accuracy_vs_tight_oracle(native_lib, oracle_mod, cuda, cfgname, n, sides):
    """Mixed precision (FP32 Jacobian/LU preconditioner, FP64 rates, residual, error test and
    step control) takes different Newton iterates than the FP64 path, so it is judged the way
    the benchmark definition asks: by its error against a tight-tolerance oracle (rtol 1e-11),
    which must be no worse than the error the plain FP64 oracle itself makes at the same
    rtol/atol (T and mass fractions: 99th percentile within 1.25x; worst cell within 2x plus
    50 rtol)."""
    torch = cuda
    cfg = CONFIGS[cfgname]
    cs, g, o, nfail = _run_both(torch, oracle_mod, cfg, n, 7, "mixed", sides)
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    tight = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, 1e-11, 1e-16,
                     max_steps=200000)
    Yt = tight[0] / tight[0].sum(1, keepdims=True)

    def errs(rY, T):
        Y = rY / rY.sum(1, keepdims=True)
        dT = np.abs(T - tight[1])
        dY = np.abs(Y - Yt).max(1)
        return dT.max(), np.percentile(dT, 99), dY.max(), np.percentile(dY, 99)

    em = errs(g[0], g[1])
    eo = errs(o[0], o[1])
    _report(f"mixed_vs_tight[{cfgname}]", {"mixed": [float(x) for x in em],
                                           "oracle_same_rtol": [float(x) for x in eo]})
    assert nfail == 0
    # 99th percentile (the distribution): within 25% of the FP64 oracle's; max over cells (a
    # single cell may take another step sequence): within 2x plus 50 rtol (relative), inside
    # the global-error envelope the FP64 method itself shows at this rtol
    Tmax = float(np.max(tight[1]))
    bounds = ((2.0, 50 * cfg.rtol * Tmax), (1.25, 1e-3), (2.0, 50 * cfg.rtol), (1.25, 1e-8))
    for a, b, (fac, slack) in zip(em, eo, bounds):
        assert a <= fac * b + slack, (em, eo)


@pytest.mark.gpu
def test_react_boxes_ghosts_offsets_mask_graph(native_lib, oracle_mod, cuda):
    """Several boxes (uneven sizes, non-zero lo, ghost cells, a mask) in one persistent launch,
    also replayed from a captured CUDA graph; covered cells keep their state and get FC = 0."""
    torch = cuda
    cfg = CONFIGS["lidryer_amr120"]
    shapes = [(8, 8, 8), (16, 4, 8), (5, 7, 3), (12, 6, 4)]
    n = sum(a * b * c for a, b, c in shapes)
    cs = make_cells(cfg, n, seed=3)
    rng = np.random.default_rng(5)
    cs.mask[:] = np.where(rng.uniform(size=n) < 0.1, -1, 1)
    los = [(0, 0, 0), (8, -4, 2), (-3, 5, 100), (40, 40, 40)]
    stream = torch.cuda.Stream()
    for graph in (0, 1):
        boxes = boxes_from_cells(torch, cs, shapes, lo_list=los, ghost=2, with_mask=True)
        r = ReactorBase.create("ReactorCvode", cfg.mech,
                               f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.graph={graph} "
                               "gb.precision=fp64")
        r.init(2, 1)
        with torch.cuda.stream(stream):
            r.react_boxes(boxes, cfg.dt, 0.0, stream=stream)
            if graph:  # second replay of the captured graph on fresh inputs
                boxes = boxes_from_cells(torch, cs, shapes, lo_list=los, ghost=2, with_mask=True)
                r.react_boxes(boxes, cfg.dt, 0.0, stream=stream)
        st = r.stats()
        stream.synchronize()
        rYg, Tg, rEg, FCg = gather(boxes, cs.rY.shape[1])
        om = oracle_mod.OracleMech(mech_path(cfg.mech))
        rYo, To, rEo, FCo, nf = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt,
                                         cfg.rtol, cfg.atol)
        covered = cs.mask < 0
        assert st["nfail"] == 0 and nf == 0
        assert st["ncell"] == n
        assert np.all(FCg[covered] == 0) and np.all(FCg[~covered] > 0)
        np.testing.assert_array_equal(Tg[covered], cs.T[covered])
        np.testing.assert_array_equal(rYg[covered], cs.rY[covered])
        relT = np.abs(Tg - To) / To
        assert relT.max() <= 1e-6
        assert tol_ratio(rYg, rYo, cfg.rtol, cfg.atol).max() <= 1.0
        r.close()


@pytest.mark.gpu
def test_null_reactor(native_lib, cuda):
    """ReactorNull advances the forcing only: rhoY += dt F, rho h += dt F_h, FC = 0."""
    torch = cuda
    cfg = CONFIGS["lidryer_amr120"]
    cs = make_cells(cfg, 512, seed=9)
    boxes = boxes_from_cells(torch, cs, [8])
    r = ReactorBase.create("ReactorNull", cfg.mech, "")
    r.init(2, 1)
    b = boxes[0]
    assert r.react(b.box, b.rY, b.rY_src, b.T, b.rEner, b.rEner_src, b.FC, None, cfg.dt, 0.0) == 0
    rYg, Tg, rEg, FCg = gather(boxes, cs.rY.shape[1])
    np.testing.assert_allclose(rYg, cs.rY + cfg.dt * cs.rYsrc, rtol=1e-14, atol=1e-30)
    np.testing.assert_allclose(rEg, cs.rE + cfg.dt * cs.rEsrc, rtol=1e-14)
    assert np.all(FCg == 0)
    r.close()


@pytest.mark.gpu
@pytest.mark.parametrize("mapping", ["thread", "warp"])
def test_advance_chemistry_mks_matches_cgs_react_and_reference_passes(native_lib, cuda, mapping):
    """pgb_advance_chemistry on MKS arrays (scaling, advance, back-scaling, I_R in the kernels)
    against the caller's own passes around react_boxes, as advance_chemistry does them
    (Source/PeleLM.cpp:5736-5801): rhoY *= 1e-3, rhoH *= 10 (and their forcing), react, rhoY *=
    1e3, rhoH *= 0.1, I_R = -(rhoY_old - rhoY_new) / dt - F. Same arithmetic: bit for bit."""
    torch = cuda
    cfg = CONFIGS["lidryer_amr120"]
    n = 4096
    cs = make_cells(cfg, n, seed=17)
    rng = np.random.default_rng(2)
    cs.mask[:] = np.where(rng.uniform(size=n) < 0.05, -1, 1)
    mks = make_cells(cfg, n, seed=17)  # the same state in MKS units
    mks.rY, mks.rYsrc, mks.rE, mks.rEsrc = cs.rY * 1e3, cs.rYsrc * 1e3, cs.rE * 0.1, cs.rEsrc * 0.1
    mks.mask[:] = cs.mask
    opts = f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.mapping={mapping}"
    # (a) caller's passes around the CGS react
    a = boxes_from_cells(torch, mks, [16], with_mask=True)[0]
    old = a.rY.clone()
    a.rY.mul_(1.0e-3); a.rY_src.mul_(1.0e-3); a.rEner.mul_(10.0); a.rEner_src.mul_(10.0)
    r = ReactorBase.create("ReactorCvode", cfg.mech, opts)
    r.init(2, 1)
    r.react_boxes([a], cfg.dt, 0.0)
    a.rY.mul_(1.0e3); a.rEner.mul_(0.1)
    src = torch.tensor(np.ascontiguousarray(mks.rYsrc.T.reshape(a.rY.shape)), device="cuda")
    IR_a = -(old - a.rY) * (1.0 / cfg.dt) - src
    # (b) fused
    b = boxes_from_cells(torch, mks, [16], with_mask=True)[0]
    IR_b = torch.zeros_like(b.rY)
    r.advance_chemistry([b], cfg.dt, I_R=[IR_b])
    torch.cuda.synchronize()
    r.close()
    cov = torch.tensor(cs.mask.reshape(16, 16, 16) < 0, device="cuda")
    for x, y in ((a.rY, b.rY), (a.T, b.T), (a.rEner, b.rEner), (a.FC, b.FC)):
        assert torch.equal(x[:, ~cov], y[:, ~cov])
    # covered cells: the fused path leaves the caller's values untouched (the caller's passes
    # scale them down and up, x * 1e-3 * 1e3, which need not round-trip exactly)
    b0 = boxes_from_cells(torch, mks, [16], with_mask=True)[0]
    for x, y in ((b0.rY, b.rY), (b0.T, b.T), (b0.rEner, b.rEner)):
        assert torch.equal(x[:, cov], y[:, cov])
    assert torch.equal(IR_a[:, ~cov], IR_b[:, ~cov])
    assert torch.equal(IR_b[:, cov], -src[:, cov])


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_reference_gpu_deck_typical_values(native_lib, oracle_mod, cuda, precision):
    """The reactor settings of the reference's GPU deck (Exec/RegTests/FlameSheet/
    inputs.3d-regt_GPU:85-89): peleLM.use_typ_vals_chem = 1, ode.rtol = 1e-6, ode.atol = 1e-5 as a
    factor on the typical values, cvode.solve_type = GMRES (run as the dense direct Newton solve),
    cvode.max_order = 4. The typical values are computed from the state as PeleLM does
    (Source/PeleLM.cpp:1497-1545) and passed through set_typ_vals_ode; the oracle gets the same
    per-component absolute tolerances ode.atol * typ. FP64: T within 1e-6 relative and rhoY within
    atol_k + rtol |rhoY| cell by cell; mixed: error against a tight oracle no worse than the
    oracle's own at the deck's tolerances."""
    from pelelm_gb300.reactor import typical_values_chem
    torch = cuda
    cfg = CONFIGS["drm19_2M"]
    n = 4096
    cs = make_cells(cfg, n, seed=31)
    typ = np.array(typical_values_chem(cs.rY * 1e3, cs.T))
    atol = 1.0e-5 * typ
    rtol = 1.0e-6
    boxes = boxes_from_cells(torch, cs, [16])
    r = ReactorBase.create("ReactorCvode", cfg.mech,
                           "peleLM.use_typ_vals_chem = 1; ode.rtol = 1.0e-6; ode.atol = 1.0e-5; "
                           f"cvode.solve_type = GMRES; cvode.max_order = 4; gb.precision = {precision}"
                           .replace(" = ", "="))
    r.init(2, 1)
    r.set_typ_vals_ode(list(typ))
    b = boxes[0]
    nfail = r.react(b.box, b.rY, b.rY_src, b.T, b.rEner, b.rEner_src, b.FC, None, cfg.dt, 0.0)
    r.close()
    rYg, Tg, rEg, FCg = gather(boxes, cs.rY.shape[1])
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    rYo, To, rEo, FCo, nf = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, rtol, atol,
                                     max_order=4)
    ns = cs.rY.shape[1]
    ratio = np.abs(rYg - rYo) / (atol[None, :ns] + rtol * np.abs(rYo))
    relT = np.abs(Tg - To) / To
    _report(f"gpu_deck_typvals[{precision}]", {
        "max_relT": float(relT.max()), "max_ratio": float(ratio.max()),
        "frac_same_nfe": float(np.mean(FCg == FCo)), "nfe_gpu": float(FCg.mean()), "nfe_orc": float(FCo.mean()),
        "atol_T": float(atol[ns]), "atol_rY_min": float(atol[:ns].min()), "atol_rY_max": float(atol[:ns].max())})
    assert nfail == 0 and nf == 0 and np.all(FCg > 0)
    np.testing.assert_allclose(rEg, rEo, rtol=1e-14, atol=1e-14 * np.abs(rEo).max())
    if precision == "fp64":
        assert relT.max() <= 1e-6, relT.max()
        assert ratio.max() <= 1.0, ratio.max()
        return
    tight = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, 1e-11, 1e-16, max_steps=200000)
    Yt = tight[0] / tight[0].sum(1, keepdims=True)

    def errs(rY, T):
        Y = rY / rY.sum(1, keepdims=True)
        dT = np.abs(T - tight[1])
        dY = np.abs(Y - Yt).max(1)
        return dT.max(), np.percentile(dT, 99), dY.max(), np.percentile(dY, 99)

    em, eo = errs(rYg, Tg), errs(rYo, To)
    Tmax = float(np.max(tight[1]))
    bounds = ((2.0, 50 * rtol * Tmax), (1.25, 1e-3), (2.0, 50 * rtol), (1.25, 1e-8))
    for a, c, (fac, slack) in zip(em, eo, bounds):
        assert a <= fac * c + slack, (em, eo)


@pytest.mark.gpu
def test_react_boxes_full_amr120_layout(native_lib, oracle_mod, cuda):
    """The whole LiDryer-shaped AMR workload as the benchmark defines it: 120 boxes with sides
    from {8, 16, 32, 64} (2,154,496 cells, nonzero forcing, dt_react 1e-5 s) in one persistent
    launch from a CUDA graph, FP64, every cell against the oracle at the same rtol/atol."""
    torch = cuda
    cfg = CONFIGS["lidryer_amr120"]
    cs = make_cells(cfg, seed=5)
    boxes = boxes_from_cells(torch, cs, cfg.boxes)
    stream = torch.cuda.Stream()
    r = ReactorBase.create("ReactorCvode", cfg.mech,
                           f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.precision=fp64 gb.graph=1")
    r.init(2, 1)
    with torch.cuda.stream(stream):
        r.react_boxes(boxes, cfg.dt, 0.0, stream=stream)
    st = r.stats()
    stream.synchronize()
    r.close()
    rYg, Tg, rEg, FCg = gather(boxes, cs.rY.shape[1])
    del boxes
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    rYo, To, rEo, FCo, nf = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt, cfg.rtol, cfg.atol)
    relT = np.abs(Tg - To) / To
    ratio = tol_ratio(rYg, rYo, cfg.rtol, cfg.atol).max(1)
    _report("react[lidryer_amr120,full layout,fp64]", {
        "cells": int(cs.T.size), "boxes": len(cfg.boxes), "max_relT": float(relT.max()),
        "max_ratio": float(ratio.max()), "frac_same_nfe": float(np.mean(FCg == FCo)),
        "nfe_gpu": float(FCg.mean()), "nfe_orc": float(FCo.mean()), "max_steps_cell": int(st["max_nst"]),
        "frac_within_plain_tol": float(np.mean((relT <= 1e-6) & (ratio <= 1.0)))})
    assert st["ncell"] == cs.T.size and st["nfail"] == 0 and nf == 0 and np.all(FCg > 0)
    np.testing.assert_allclose(rEg, rEo, rtol=1e-14, atol=1e-14 * np.abs(rEo).max())
    within = (relT <= 1e-6) & (ratio <= 1.0)
    assert within.mean() >= 0.999, within.mean()
    # a cell outside the plain tolerances has taken another step sequence (the generated rate
    # code and the oracle's table code may differ in the last bit): it is held to the oracle's
    # own error on that cell against a tight oracle (rtol 1e-11), at most 2x plus 50 rtol
    out = np.nonzero(~within)[0]
    outliers_within_global_error(om, cs, out, (rYg[out], Tg[out]), (rYo[out], To[out]), cfg.dt, cfg.rtol)
