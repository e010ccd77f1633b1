"""GPU tests of the learned surrogate with BDF fallback on the drm19-shaped mechanism.

The trained file (pelelm_gb300/data/drm19_syn.pgbs) comes from pelelm_gb300.surrogate_train on
the drm19_2M workload distribution (seed 11); these tests draw other cells (seed 4242) from the
same distribution. What is checked:
  * cells the surrogate rejects (and the audit sample) are advanced by the BDF bit for bit as
    the plain reactor advances them;
  * accepted cells are within 1 K and 1e-4 (mass fraction) of the FP64 oracle at rtol 1e-10
    and of the plain GPU BDF;
  * accepted cells conserve mass and elements exactly (to round-off), carry rhoH + dt F_h, and
    their T solves h(T) = rhoH / rho;
  * the fused inference kernel reproduces the unfused network (the training kernels) and the
    FP64 restatement of its update (surrogate_train.apply_prediction);
  * the audit sample, its error report, masks, ghost cells, graph replay, bad files.
"""
import os
import time

import numpy as np
import pytest

from helpers import boxes_from_cells, gather

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SURR = os.path.join(ROOT, "pelelm_gb300", "data", "drm19_syn.pgbs")
TOL_T, TOL_Y = 1.0, 1e-4
ACCEPT_ALL = ("gb.sg.mis=1e30 gb.sg.cons=1e30 gb.sg.disT=1e30 gb.sg.disY=1e30 gb.sg.neg=1e30 "
              "gb.sg.ood_margin=1e30")


def _report(name, d):
    import json
    out = os.environ.get("PGB_TEST_OUT", os.path.join(ROOT, "test_reports"))
    os.makedirs(out, exist_ok=True)
    with open(os.path.join(out, "surrogate_tests.jsonl"), "a") as f:
        f.write(json.dumps({"test": name, **d}) + "\n")


def _run(torch, cfg, cs, sides, opts, ghost=0, lo=None, mask=False, stream=None, calls=1):
    from pelelm_gb300.reactor import ReactorBase
    r = ReactorBase.create("ReactorCvode", cfg.mech, opts)
    r.init(2, 1)
    outs = []
    boxes = boxes_from_cells(torch, cs, sides, lo_list=lo, ghost=ghost, with_mask=mask)
    pristine = [[t.clone() for t in (b.rY, b.T, b.rEner, b.FC)] for b in boxes]
    for call in range(calls):
        if call:  # same buffers (a graph replays), initial contents
            for b, p in zip(boxes, pristine):
                for t, q in zip((b.rY, b.T, b.rEner, b.FC), p):
                    t.copy_(q)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.react_boxes(boxes, cfg.dt, 0.0, stream=stream)
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        st = r.stats()
        sst = r.surrogate_stats() if "gb.surrogate" in opts else None
        outs.append((gather(boxes, cs.rY.shape[1]), st, sst, dt))
    r.close()
    return outs if calls > 1 else outs[0]


def levels():
    """Operating points calibrated at training time (tolerance -> gate thresholds)."""
    import json
    with open(SURR + ".levels.json") as f:
        return json.load(f)["levels"]


def level_opts(lv):
    return " ".join(f"gb.sg.{k}={lv[k]!r}" for k in ("mis", "cons", "disT", "disY", "neg", "tol_T", "tol_Y"))


def loose_level():
    """The tightest calibrated operating point that accepts at least 5% of validation cells."""
    for lv in levels():
        if lv["val_accept"] >= 0.05:
            return lv
    return levels()[-1]


@pytest.fixture(scope="module")
def drm19(native_lib, cuda):
    from pelelm_gb300.workloads import CONFIGS, make_cells
    cfg = CONFIGS["drm19_2M"]
    n = 8 * 16 ** 3
    cs = make_cells(cfg, n, seed=4242)
    base = f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.precision=mixed"
    sides = [16] * 8
    lv = loose_level()
    plain = _run(cuda, cfg, cs, sides, base)
    surr = _run(cuda, cfg, cs, sides, base + f" gb.surrogate={SURR}")
    loose = _run(cuda, cfg, cs, sides, base + f" gb.surrogate={SURR} " + level_opts(lv))
    return dict(cfg=cfg, cs=cs, base=base, sides=sides, plain=plain, surr=surr, loose=loose, level=lv)


def _Y(rY):
    return rY / rY.sum(1, keepdims=True)


def _check_fallback_and_accepted(gp, gs, sst, tol_T, tol_Y, name):
    n = gp[0].shape[0]
    acc = gs[3] == 0.0
    assert sst["ncell"] == n
    assert sst["accept"] == int(acc.sum())
    assert sst["accept"] + sst["fallback"] == n
    fb = ~acc
    assert np.array_equal(gs[0][fb], gp[0][fb]) and np.array_equal(gs[1][fb], gp[1][fb])
    assert np.array_equal(gs[3][fb], gp[3][fb])
    rep = {"ncell": n, "accept": int(acc.sum()), "tol_T": tol_T, "tol_Y": tol_Y, "sst": sst}
    if acc.any():
        eT = np.abs(gs[1] - gp[1])[acc]
        eY = np.abs(_Y(gs[0]) - _Y(gp[0])).max(1)[acc]
        rep.update(max_eT=float(eT.max()), max_eY=float(eY.max()))
        assert eT.max() <= tol_T and eY.max() <= tol_Y
    _report(name, rep)
    return acc


@pytest.mark.gpu
def test_default_gates_fallback_is_plain_bdf_and_accepted_cells_within_1K(drm19):
    """The file's own gates (calibrated for 1 K / 1e-4): whatever they accept is within those
    tolerances of the plain BDF; every other cell is the plain BDF's result, bit for bit."""
    _check_fallback_and_accepted(drm19["plain"][0], drm19["surr"][0], drm19["surr"][2], TOL_T, TOL_Y,
                                 "default_gates_vs_plain_bdf")


@pytest.mark.gpu
def test_looser_operating_point_accepts_cells_within_its_tolerance(drm19, oracle_mod):
    """A looser calibrated operating point accepts cells; they stay within its tolerances of
    the plain BDF and of the FP64 oracle at rtol 1e-10."""
    from pelelm_gb300.workloads import mech_path
    lv = drm19["level"]
    cfg, cs = drm19["cfg"], drm19["cs"]
    gs, _, sst, _ = drm19["loose"]
    acc = _check_fallback_and_accepted(drm19["plain"][0], gs, sst, lv["tol_T"], lv["tol_Y"],
                                       "loose_gates_vs_plain_bdf")
    assert acc.mean() > 0.01, "the looser operating point accepts (almost) no cell"
    idx = np.nonzero(acc)[0]
    idx = idx[np.linspace(0, idx.size - 1, min(idx.size, 1024)).astype(int)]
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    tight = om.react(cs.rY[idx], cs.rYsrc[idx], cs.T[idx], cs.rE[idx], cs.rEsrc[idx], cs.mask[idx], cfg.dt,
                     1e-10, 1e-14, max_steps=200000)
    eT = np.abs(gs[1][idx] - tight[1])
    eY = np.abs(_Y(gs[0][idx]) - _Y(tight[0])).max(1)
    _report("loose_accepted_vs_tight_oracle", {"n": int(idx.size), "tol_T": lv["tol_T"], "tol_Y": lv["tol_Y"],
                                               "max_eT": float(eT.max()), "max_eY": float(eY.max())})
    assert eT.max() <= lv["tol_T"] and eY.max() <= lv["tol_Y"]


@pytest.mark.gpu
def test_accepted_cells_conserve_mass_elements_enthalpy(drm19, oracle_mod):
    from pelelm_gb300.surrogate import read_pgbs
    from pelelm_gb300.workloads import mech_path
    cfg, cs = drm19["cfg"], drm19["cs"]
    gs = drm19["loose"][0]
    acc = gs[3] == 0.0
    assert acc.any()
    d = read_pgbs(SURR)
    rY0, F = cs.rY[acc], cs.rYsrc[acc]
    rY1 = gs[0][acc]
    mass0 = (rY0 + cfg.dt * F).sum(1)
    assert np.abs(rY1.sum(1) - mass0).max() <= 1e-12 * mass0.max()
    rho0 = rY0.sum(1, keepdims=True)
    dchem = (rY1 - rY0 - cfg.dt * F) / rho0
    viol = dchem @ d["A"].T                      # element moles per gram, per element
    scale = np.abs(dchem) @ np.abs(d["A"]).T + 1e-300
    assert (np.abs(viol) / scale).max() <= 1e-9
    np.testing.assert_allclose(gs[2][acc], cs.rE[acc] + cfg.dt * cs.rEsrc[acc], rtol=1e-14, atol=1e-14)
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    rho1 = rY1.sum(1)
    T = om.hy2t(gs[2][acc] / rho1, rY1 / rho1[:, None], gs[1][acc])
    assert np.abs(T - gs[1][acc]).max() <= 1e-7 * T.max()


@pytest.mark.gpu
def test_reject_all_is_the_plain_bdf(drm19, cuda):
    gp = drm19["plain"][0]
    g, _, sst, _ = _run(cuda, drm19["cfg"], drm19["cs"], drm19["sides"],
                        drm19["base"] + f" gb.surrogate={SURR} gb.sg.mis=-1")
    assert sst["accept"] == 0 and sst["fallback"] == sst["ncell"] == gp[0].shape[0]
    for a, b in zip(g, gp):
        assert np.array_equal(a, b)


@pytest.mark.gpu
def test_fused_kernel_matches_unfused_network_and_fp64_update(drm19, cuda):
    """All gates open, no audit: every cell takes the surrogate's update. The same update is
    computed from the unfused network (the training GEMM kernels) and the FP64 restatement."""
    from pelelm_gb300.surrogate import models_from_pgbs, read_pgbs
    from pelelm_gb300.surrogate_train import Thermo, apply_prediction, normalise, raw_features
    from pelelm_gb300.workloads import load_mechanism
    torch = cuda
    cfg, cs = drm19["cfg"], drm19["cs"]
    g, _, sst, _ = _run(torch, cfg, cs, drm19["sides"],
                        drm19["base"] + f" gb.surrogate={SURR} gb.sg.audit=0 " + ACCEPT_ALL)
    n = g[0].shape[0]
    assert sst["accept"] == n and sst["fallback"] == 0
    assert np.all(g[3] == 0.0)
    d = read_pgbs(SURR)
    models = models_from_pgbs(torch, d)
    dev = lambda a: torch.tensor(np.asarray(a), device="cuda")  # noqa: E731
    st = dict(rY0=dev(cs.rY), F=dev(cs.rYsrc), rE0=dev(cs.rE), Fh=dev(cs.rEsrc), T0=dev(cs.T))
    from pelelm_gb300.surrogate import surrogate_features
    x = surrogate_features(torch, cfg.mech, boxes_from_cells(torch, cs, drm19["sides"]))
    xt = raw_features(torch, st["rY0"], st["T0"], st["F"], st["Fh"])
    # the torch restatement of the featurisation agrees to a few FP32 ulps (log10 differs)
    assert torch.allclose(x, xt, rtol=1e-6, atol=1e-6)
    X = models[0].prepare_input(normalise(torch, x, d["x_mean"], d["x_std"]))
    # raw network: the fused kernel's input rows and both members' outputs equal the training
    # kernels' bit for bit
    from pelelm_gb300.reactor import ReactorBase
    rr = ReactorBase.create("ReactorCvode", cfg.mech, f"gb.surrogate={SURR}")
    rr.init(2, 1)
    raw = torch.empty(n, d["nmodel"], d["n_out"], device="cuda")
    rin = torch.empty(n, d["k_in"], device="cuda")
    rr.surrogate_raw(boxes_from_cells(torch, cs, drm19["sides"]), raw, rin)
    torch.cuda.synchronize()
    rr.close()
    assert torch.equal(rin, X.float())
    preds = [m.forward(X)[:, :d["n_out"]] for m in models]
    for mi, p in enumerate(preds):
        assert torch.equal(raw[:, mi, :], p), mi
    preds = [p.double() for p in preds]
    u = apply_prediction(torch, Thermo(torch, load_mechanism(cfg.mech)), st, preds, d["y_scale"],
                         d["out_species"], d["A"], d["P"], cfg.dt)
    dT = np.abs(u["T"].cpu().numpy() - g[1])
    dY = np.abs(u["Y1"].cpu().numpy() - _Y(g[0])).max(1)
    _report("fused_vs_unfused", {"p999_dT": float(np.percentile(dT, 99.9)), "max_dT": float(dT.max()),
                                 "p999_dY": float(np.percentile(dY, 99.9)), "max_dY": float(dY.max())})
    # the same features, the same BF16 products in the same order: the network outputs agree
    # bit for bit and the FP64 update to round-off (HY2T iterates, ensemble-mean order)
    assert (dT <= 1e-6).mean() >= 0.999 and (dY <= 1e-10).mean() >= 0.999
    assert dT.max() <= 1e-3 and dY.max() <= 1e-6


@pytest.mark.gpu
def test_audit_sample_is_bdf_and_reports_surrogate_error(drm19, cuda):
    torch = cuda
    cfg, cs = drm19["cfg"], drm19["cs"]
    gp = drm19["plain"][0]
    base = drm19["base"] + f" gb.surrogate={SURR} " + ACCEPT_ALL
    g_all, _, _, _ = _run(torch, cfg, cs, drm19["sides"], base + " gb.sg.audit=0")
    g, _, sst, _ = _run(torch, cfg, cs, drm19["sides"], base + " gb.sg.audit=0.1 gb.sg.seed=7")
    n = gp[0].shape[0]
    aud = g[3] != 0.0
    assert sst["audit"] == int(aud.sum()) == sst["fallback"]
    assert abs(sst["audit"] - 0.1 * n) <= 5.0 * np.sqrt(0.1 * 0.9 * n)
    assert np.array_equal(g[0][aud], gp[0][aud]) and np.array_equal(g[1][aud], gp[1][aud])
    assert np.array_equal(g[0][~aud], g_all[0][~aud])
    eT = np.abs(g_all[1][aud] - gp[1][aud])
    eY = np.abs(_Y(g_all[0][aud]) - _Y(gp[0][aud])).max(1)
    assert sst["audit_max_dT"] == pytest.approx(float(eT.max()), rel=1e-12, abs=1e-12)
    assert sst["audit_max_dY"] == pytest.approx(float(eY.max()), rel=1e-12, abs=1e-15)
    assert sst["audit_bad"] == int(((eT > TOL_T) | (eY > TOL_Y)).sum())


@pytest.mark.gpu
def test_masked_ghosted_offset_boxes_and_graph_replay(drm19, cuda):
    torch = cuda
    cfg, cs = drm19["cfg"], drm19["cs"]
    base = drm19["base"] + f" gb.surrogate={SURR} gb.sg.audit=0"
    ref = _run(torch, cfg, cs, drm19["sides"], base)[0]
    cs.mask[::7] = -1
    try:
        lo = [(16 * b, -3, 5) for b in range(8)]
        stream = torch.cuda.Stream()
        runs = _run(torch, cfg, cs, drm19["sides"], base + " gb.graph=1", ghost=1, lo=lo, mask=True,
                    stream=stream, calls=2)
    finally:
        cs.mask[::7] = 1
    for g, _, sst, _ in runs:
        m = np.zeros(cs.T.size, dtype=bool)
        m[::7] = True
        assert np.array_equal(g[0][m], cs.rY[m]) and np.array_equal(g[1][m], cs.T[m])
        assert np.all(g[3][m] == 0.0)
        assert sst["ncell"] == int((~m).sum())
        for a, b in zip(g, ref):
            assert np.array_equal(a[~m], b[~m])


@pytest.mark.gpu
def test_graph_replay_draws_a_new_audit_sample(drm19, cuda):
    torch = cuda
    stream = torch.cuda.Stream()
    runs = _run(torch, drm19["cfg"], drm19["cs"], drm19["sides"],
                drm19["base"] + f" gb.surrogate={SURR} gb.graph=1 gb.sg.audit=0.05 " + ACCEPT_ALL,
                stream=stream, calls=2)
    a0, a1 = runs[0][0][3] != 0.0, runs[1][0][3] != 0.0
    assert a0.sum() > 0 and a1.sum() > 0 and not np.array_equal(a0, a1)


@pytest.mark.gpu
def test_bad_surrogate_files_are_rejected(native_lib, cuda, tmp_path):
    from pelelm_gb300.reactor import ReactorBase
    # ReactorBase::create only names the reactor; init() builds it (as in the reference)
    with pytest.raises(RuntimeError, match="another mechanism"):
        ReactorBase.create("ReactorCvode", "lidryer_syn", f"gb.surrogate={SURR}").init(2, 1)
    bad = tmp_path / "trunc.pgbs"
    bad.write_bytes(open(SURR, "rb").read()[:5000])
    with pytest.raises(RuntimeError, match="truncated"):
        ReactorBase.create("ReactorCvode", "drm19_syn", f"gb.surrogate={bad}").init(2, 1)
    with pytest.raises(RuntimeError, match="cannot open"):
        ReactorBase.create("ReactorCvode", "drm19_syn", f"gb.surrogate={tmp_path / 'missing.pgbs'}").init(2, 1)
    with pytest.raises(RuntimeError, match="ReactorCvode"):
        ReactorBase.create("ReactorNull", "drm19_syn", f"gb.surrogate={SURR}").init(2, 1)


@pytest.mark.gpu
def test_surrogate_gain_over_plain_bdf(native_lib, cuda):
    """What the trained network gains over the method without it: the same cells through the
    plain GPU BDF and through surrogate + fallback (1% audit) at every calibrated operating
    point; reported per point: accepted share, share of the BDF work (RHS evaluations) the
    accepted cells no longer need, wall-time ratio. Asserted: the surrogate pass costs little
    next to the BDF (the run is no slower than the plain BDF on the cells it still integrates,
    plus 5%), and the loosest point saves BDF work."""
    from pelelm_gb300.workloads import CONFIGS, make_cells
    torch = cuda
    cfg = CONFIGS["drm19_2M"]
    cs = make_cells(cfg, 32 * 32 ** 3, seed=4343)
    base = f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.precision=mixed"
    gp, _, _, tp = _run(torch, cfg, cs, [32] * 32, base)
    saved = []
    for lv in levels():
        gs, _, sst, ts = _run(torch, cfg, cs, [32] * 32, base + f" gb.surrogate={SURR} " + level_opts(lv))
        acc = gs[3] == 0.0
        sv = float(gp[3][acc].sum() / gp[3].sum())
        saved.append(sv)
        _report("gain", {"tol_T": lv["tol_T"], "tol_Y": lv["tol_Y"], "ncell": int(acc.size),
                         "accept": float(acc.mean()), "work_saved": sv, "plain_s": tp, "surrogate_s": ts,
                         "speedup": tp / ts, "sst": sst})
        assert ts <= 1.05 * tp * (1.0 - sv) + 0.02
        if lv["tol_T"] == TOL_T and lv["tol_Y"] == TOL_Y:
            # the benchmark's 1 K / 1e-4 point: calibrated on a million held-out cells, the gates
            # keep no cell whose error could exceed the bar, so the gain there is the plain
            # BDF's speed less the inference pass, and any accepted cell is within the bar
            _check_fallback_and_accepted(gp, gs, sst, TOL_T, TOL_Y, "gain_at_1K")
            assert tp / ts >= 0.95, f"surrogate + fallback at 1 K runs at {tp / ts:.3f} of the plain BDF"
    assert saved[-1] > 0.0
