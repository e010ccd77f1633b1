"""Reactor states from the reference's own 1-D flame profiles (tests/golden/flame_states.npz,
made by tests/golden/make_flame_states.py from Exec/RegTests/*/p*pmf*.dat): the species order of
the profiles is the mechanisms' order, and the oracle advances a spread of them (cold gas to
burnt gas, no forcing) as scipy's VODE BDF does at rtol 1e-12."""
import os

import numpy as np

from pelelm_gb300.workloads import CONFIGS, load_mechanism, mech_path, mixture_h

HERE = os.path.dirname(os.path.abspath(__file__))
G = np.load(os.path.join(HERE, "golden", "flame_states.npz"))
CFGS = ("lidryer_amr120", "drm19_2M")


def flame_cells(cfgname):
    """(rY, T, rE) of every stored flame state of a config, CGS."""
    rho, Y, T = G[f"{cfgname}/rho"], G[f"{cfgname}/Y"], G[f"{cfgname}/T"]
    return rho[:, None] * Y, T, G[f"{cfgname}/rE"]


def test_profile_species_order_is_the_mechanism_order():
    for cfgname in CFGS:
        m = load_mechanism(CONFIGS[cfgname].mech)
        assert [s.name for s in m.species] == [str(s) for s in G[f"{cfgname}/species"]]


def test_flame_states_are_physical():
    for cfgname in CFGS:
        m = load_mechanism(CONFIGS[cfgname].mech)
        rY, T, rE = flame_cells(cfgname)
        Y = rY / rY.sum(1, keepdims=True)
        assert np.all(Y >= 0.0) and np.allclose(Y.sum(1), 1.0)
        assert T.min() < 400.0 and T.max() > 1400.0 and np.all(np.diff(T) > 0.0)
        np.testing.assert_allclose(rE, rY.sum(1) * mixture_h(m, T, Y), rtol=1e-12, atol=1e-12 * np.abs(rE).max())


def test_oracle_matches_vode_on_flame_states(oracle_mod):
    for cfgname in CFGS:
        cfg = CONFIGS[cfgname]
        om = oracle_mod.OracleMech(mech_path(cfg.mech))
        rY, T, _ = flame_cells(cfgname)
        sel, yT = G[f"{cfgname}/vode_sel"], G[f"{cfgname}/vode_yT"]
        zero = np.zeros(rY.shape[1])
        for c, s in enumerate(sel):
            y, status, _ = om.bdf_one(np.append(rY[s], T[s]), zero, 0.0, float(G[f"{cfgname}/dt"]), 1e-11, 1e-20)
            assert status == 0
            assert abs(y[-1] - yT[c, -1]) <= 1e-7 * yT[c, -1], (cfgname, s, y[-1], yT[c, -1])
            assert np.max(np.abs(y[:-1] - yT[c, :-1])) <= 1e-9 * yT[c, :-1].sum(), (cfgname, s)
