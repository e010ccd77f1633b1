"""CPU pins of the oracle (no GPU): the reference ships no golden vectors for its reactor, so the
oracle is pinned by conservation laws, closed-form solutions, finite differences and an
independent compiled BDF (scipy VODE, tests/golden/vode_cells.npz)."""
import os

import numpy as np
import pytest

from pelelm_gb300.mech.model import P_ATM, R_ERG
from pelelm_gb300.workloads import CONFIGS, load_mechanism, make_cells, mech_path

HERE = os.path.dirname(os.path.abspath(__file__))
MECHS = ["lidryer_syn", "drm19_syn", "gri_syn"]
CFG_OF = {"lidryer_syn": "lidryer_amr120", "drm19_syn": "drm19_2M", "gri_syn": "gri_1M"}


def _elements(m):
    comp = np.zeros((m.ns, len(m.elements)))
    for k, s in enumerate(m.species):
        for e, n in s.composition.items():
            comp[k, m.elements.index(e)] = n
    return comp


@pytest.mark.parametrize("mech", MECHS)
def test_wdot_conserves_mass_and_elements(oracle_mod, mech):
    m = load_mechanism(mech)
    om = oracle_mod.OracleMech(mech_path(mech))
    cs = make_cells(CONFIGS[CFG_OF[mech]], 300, seed=1)
    W = np.array([s.W for s in m.species])
    wd = om.wdot(cs.T, cs.rY / W)
    scale = np.abs(wd * W).max(axis=1)
    assert np.all(np.abs((wd * W).sum(axis=1)) <= 1e-12 * scale + 1e-300)
    el = wd @ _elements(m)
    assert np.all(np.abs(el).max(axis=1) <= 1e-12 * np.abs(wd).max(axis=1) + 1e-300)


def _jac_errors(om, cs, N):
    out = []
    for c in range(cs.ncell):
        y = np.append(cs.rY[c], cs.T[c])
        F = cs.rYsrc[c]
        Fh = cs.rEsrc[c]
        J = om.jac(y, F, Fh)
        Jfd = np.zeros((N, N))
        for j in range(N):
            # step floor scaled by the density so trace species are not differenced at 1e-14
            h = max(1e-6 * abs(y[j]), 1e-9 * y[:-1].sum())
            yp, ym = y.copy(), y.copy()
            yp[j] += h
            ym[j] -= h
            Jfd[:, j] = (om.rhs(yp, F, [Fh])[0] - om.rhs(ym, F, [Fh])[0]) / (2 * h)
        # entries below 1e-4 of their row's largest are judged on that absolute scale
        rowscale = np.abs(Jfd).max(axis=1, keepdims=True) + 1e-300
        out.append(np.abs(J - Jfd) / (np.abs(Jfd) + 1e-4 * rowscale))
    return out


@pytest.mark.parametrize("mech", ["lidryer_syn", "drm19_syn"])
def test_jacobian_matches_finite_differences(oracle_mod, tmp_path, mech):
    """Analytic Jacobian vs central differences. With Lindemann falloff (Troe parameters dropped)
    the analytic form is exact; with Troe the blending factor F is held frozen in the [M] and T
    derivatives (a documented preconditioner approximation), which bounds the worst entry."""
    m = load_mechanism(mech)
    cs = make_cells(CONFIGS[CFG_OF[mech]], 6, seed=2)
    N = m.ns + 1
    om = oracle_mod.OracleMech(mech_path(mech))
    errs = _jac_errors(om, cs, N)
    assert max(e.max() for e in errs) < 0.5
    assert max(np.median(e) for e in errs) < 1e-6
    for r in m.reactions:
        r.troe = None
    p = tmp_path / f"{mech}_lindemann.mech"
    m.to_flat(str(p))
    errs = _jac_errors(oracle_mod.OracleMech(str(p)), cs, N)
    assert max(e.max() for e in errs) < 1e-3


def _two_species_mech(tmp_path, A, reversible):
    """A <=> B (or A => B) isomerisation between species with identical W and thermo: T, rho h
    and K_c = 1 stay constant, so rhoY_A relaxes exponentially (closed form)."""
    a = "3.5 0.0 0.0 0.0 0.0 -1000.0 5.0"
    lines = ["2 1 1",
             f"28.0 1000.0 {a} {a} 1 0 2",
             f"28.0 1000.0 {a} {a} 1 0 2",
             f"0 {1 if reversible else 0} 1 0 1 1 1 1 {A!r} 0.0 0.0"]
    p = tmp_path / "iso.mech"
    p.write_text("\n".join(lines) + "\n")
    return str(p)


@pytest.mark.parametrize("reversible", [False, True])
def test_bdf_closed_form_relaxation(oracle_mod, tmp_path, reversible):
    k = 3.0e5
    om = oracle_mod.OracleMech(_two_species_mech(tmp_path, k, reversible))
    rho = 1e-3
    y0 = np.array([0.9 * rho, 0.1 * rho, 1200.0])
    dt = 2e-5
    y, status, st = om.bdf_one(y0, np.zeros(2), 0.0, dt, 1e-10, 1e-18)
    assert status == 0
    if reversible:
        eq = 0.5 * rho
        exact = eq + (y0[0] - eq) * np.exp(-2 * k * dt)
    else:
        exact = y0[0] * np.exp(-k * dt)
    assert abs(y[0] - exact) <= 1e-8 * rho
    assert abs(y[0] + y[1] - rho) <= 1e-14 * rho
    assert abs(y[2] - 1200.0) <= 1e-9
    # the same problem at the benchmark tolerance is still accurate to ~rtol
    y6, status, st6 = om.bdf_one(y0, np.zeros(2), 0.0, dt, 1e-6, 1e-14)
    assert status == 0 and abs(y6[0] - exact) <= 2e-5 * rho
    assert st6[1] < st[1]  # fewer RHS evaluations at the looser tolerance


def test_oracle_matches_vode_golden(oracle_mod):
    """Tight oracle (rtol 1e-11) against scipy VODE BDF at rtol 1e-12 (committed fixture)."""
    g = np.load(os.path.join(HERE, "golden", "vode_cells.npz"))
    for cfgname in ("lidryer_32cube", "lidryer_amr120", "drm19_2M", "gri_1M"):
        cfg = CONFIGS[cfgname]
        om = oracle_mod.OracleMech(mech_path(cfg.mech))
        y0, F, Fh, yT = (g[f"{cfgname}/{k}"] for k in ("y0", "F", "Fh", "yT"))
        for c in range(y0.shape[0]):
            y, status, _ = om.bdf_one(y0[c], F[c], Fh[c], float(g[f"{cfgname}/dt"]), 1e-11, 1e-20)
            assert status == 0
            assert abs(y[-1] - yT[c, -1]) <= 1e-7 * yT[c, -1], (cfgname, c, y[-1], yT[c, -1])
            rho = yT[c, :-1].sum()
            assert np.max(np.abs(y[:-1] - yT[c, :-1])) <= 1e-9 * rho, (cfgname, c)


def test_equilibrium_rates_vanish(oracle_mod):
    """After a long adiabatic advance the mixture sits at chemical equilibrium: net production
    rates are a tiny fraction of the forward rates of progress."""
    cfg = CONFIGS["lidryer_32cube"]
    m = load_mechanism(cfg.mech)
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    cs = make_cells(cfg, 4, seed=5)
    W = np.array([s.W for s in m.species])
    for c in range(4):
        y0 = np.append(cs.rY[c], 1500.0)
        y, status, _ = om.bdf_one(y0, np.zeros(m.ns), 0.0, 1.0, 1e-10, 1e-20)
        assert status == 0
        wd = om.wdot(np.array([y[-1]]), (y[:-1] / W)[None])[0]
        # scale: the magnitude of the fastest single reaction channel, bounded below by the
        # total concentration times a collision-like frequency
        Ctot = (y[:-1] / W).sum()
        assert np.max(np.abs(wd)) <= 1e-6 * Ctot * 1e3


@pytest.mark.parametrize("mech", MECHS)
def test_hy2t_roundtrip(oracle_mod, mech):
    m = load_mechanism(mech)
    om = oracle_mod.OracleMech(mech_path(mech))
    cs = make_cells(CONFIGS[CFG_OF[mech]], 200, seed=8)
    rho = cs.rY.sum(axis=1)
    Y = cs.rY / rho[:, None]
    T = om.hy2t(cs.rE / rho, Y, np.full(200, 1000.0))
    np.testing.assert_allclose(T, cs.T, rtol=1e-9)


def test_react_conserves_enthalpy_and_mass(oracle_mod):
    """rho h advances exactly by F_h dt; with zero net species forcing total mass is kept."""
    cfg = CONFIGS["lidryer_amr120"]
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    cs = make_cells(cfg, 256, seed=4)
    rY, T, rE, FC, nfail = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt,
                                    cfg.rtol, cfg.atol)
    assert nfail == 0 and np.all(FC > 0)
    np.testing.assert_allclose(rE, cs.rE + cfg.dt * cs.rEsrc, rtol=1e-14)
    np.testing.assert_allclose(rY.sum(axis=1), cs.rY.sum(axis=1), rtol=1e-9)


def test_react_skips_masked_cells(oracle_mod):
    cfg = CONFIGS["lidryer_32cube"]
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    cs = make_cells(cfg, 64, seed=6)
    cs.mask[::3] = -1
    rY, T, rE, FC, nfail = om.react(cs.rY, cs.rYsrc, cs.T, cs.rE, cs.rEsrc, cs.mask, cfg.dt,
                                    cfg.rtol, cfg.atol)
    assert np.all(FC[::3] == 0)
    np.testing.assert_array_equal(rY[::3], cs.rY[::3])
    np.testing.assert_array_equal(T[::3], cs.T[::3])


def test_op_count_model_matches_counting_oracle(oracle_mod):
    from pelelm_gb300.mech.opcount import rhs_ops
    for mech in MECHS:
        m = load_mechanism(mech)
        om = oracle_mod.OracleMech(mech_path(mech))
        y = np.append(np.full(m.ns, 1e-5), 1500.0)
        assert om.count_rhs(y, np.zeros(m.ns), 0.0) == rhs_ops(m)


def test_lu_known_answers(oracle_mod):
    """The integrator's partial-pivot LU: residuals at round-off on random systems of the three
    mechanisms' sizes and on Newton matrices I - gamma J of a real cell, exact answers where
    pivoting is forced (zero diagonal), and singular matrices reported."""
    rng = np.random.default_rng(17)
    for n in (10, 22, 54):
        A = rng.normal(size=(n, n)) + n * np.eye(n) * rng.uniform(0.0, 1.0)
        b = rng.normal(size=n)
        x = oracle_mod.lu_solve(A, b)
        assert np.linalg.norm(A @ x - b) <= 1e-13 * np.linalg.norm(A) * np.linalg.norm(x)
        np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-9, atol=1e-12 * np.abs(x).max())
    # a permutation with a zero diagonal: exact
    P = np.eye(6)[[3, 0, 5, 1, 2, 4]]
    assert np.all(np.diag(P) == 0.0)
    b = np.arange(1.0, 7.0)
    np.testing.assert_array_equal(oracle_mod.lu_solve(P, b), P.T @ b)
    # a zero column, and an all-zero matrix: singular
    S = rng.normal(size=(5, 5))
    S[:, 2] = 0.0
    assert oracle_mod.lu_solve(S, np.ones(5)) is None
    assert oracle_mod.lu_solve(np.zeros((3, 3)), np.ones(3)) is None
    # Newton matrices of a drm19 cell over the step sizes the integrator takes
    cfg = CONFIGS["drm19_2M"]
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    cs = make_cells(cfg, 1, seed=23)
    y = np.append(cs.rY[0], cs.T[0])
    J = om.jac(y, cs.rYsrc[0], cs.rEsrc[0])
    for gamma in (1e-10, 1e-8, 1e-6):
        M = np.eye(y.size) - gamma * J
        b = rng.normal(size=y.size)
        x = oracle_mod.lu_solve(M, b)
        assert np.linalg.norm(M @ x - b) <= 1e-12 * np.linalg.norm(M) * np.linalg.norm(x)
