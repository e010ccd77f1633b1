"""Generates tests/golden/flame_states.npz: reactor input states taken from the reference's own
1-D premixed flame profiles, plus VODE advances of a few of them.

The reference ships two flame profiles with the species orders of its LiDryer and drm19
mechanisms (Exec/RegTests/EB_FlamePastCylinder/pmf_040_01Atm.dat, 921 points, and
Exec/RegTests/FlameSheet/drm19_pmf.dat, 2048 points; columns X, temp, u, rho [g/cm^3], then one
mass fraction per species). They are the most realistic states the reference holds for its
chemistry path: cold reactants, the preheat zone, radical-rich reaction zone and burnt gas.
This script takes up to `NSTATE` points whose temperatures are evenly spaced between the cold
and burnt ends (both profiles are monotone in T, and most of their points are burnt gas), clips
the round-off negative mass fractions of the profiles to zero and renormalises, and stores T, Y
and rho per point together with the species names of the header (the tests check them against
the mechanisms' species order). For `NVODE` of the points it also stores an advance over the
workload's dt_react without forcing, computed by scipy's VODE BDF at rtol 1e-12 on the oracle's
right-hand side and analytic Jacobian (the same independent pin as make_golden.py).

    python tests/golden/make_flame_states.py <PeleLM source tree>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from make_golden import vode_cell  # noqa: E402
from pelelm_gb300.workloads import CONFIGS, load_mechanism, mech_path, mixture_h  # noqa: E402

NSTATE = 192
NVODE = 8
PROFILES = {
    # mechanism config -> profile file within the reference tree
    "lidryer_amr120": "Exec/RegTests/EB_FlamePastCylinder/pmf_040_01Atm.dat",
    "drm19_2M": "Exec/RegTests/FlameSheet/drm19_pmf.dat",
}


def read_profile(path):
    with open(path) as f:
        head = f.readline()
        names = [s.strip('"') for s in head.split("=", 1)[1].split()]
        f.readline()  # ZONE line
        data = np.loadtxt(f)
    return names, data


def main():
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_flame_states.py <PeleLM source tree>")
    ref = sys.argv[1]
    out = {}
    for cfgname, rel in PROFILES.items():
        cfg = CONFIGS[cfgname]
        mech = load_mechanism(cfg.mech)
        names, data = read_profile(os.path.join(ref, rel))
        assert names[:4] == ["X", "temp", "u", "rho"], names[:4]
        sp = names[4:]
        Tp = data[:, 1]
        assert np.all(np.diff(Tp) >= 0.0), "profile not monotone in T"
        idx = np.unique(np.minimum(np.searchsorted(Tp, np.linspace(Tp[0], Tp[-1], NSTATE)), len(Tp) - 1))
        T = data[idx, 1]
        rho = data[idx, 3]
        Y = np.clip(data[idx, 4:], 0.0, None)
        Y /= Y.sum(axis=1, keepdims=True)
        rY = rho[:, None] * Y
        rE = rho * mixture_h(mech, T, Y)
        out[f"{cfgname}/species"] = np.array(sp)
        out[f"{cfgname}/x"] = data[idx, 0]
        out[f"{cfgname}/T"] = T
        out[f"{cfgname}/rho"] = rho
        out[f"{cfgname}/Y"] = Y
        # VODE advances of NVODE points spread over the profile (no forcing)
        om = O.OracleMech(mech_path(cfg.mech))
        sel = np.linspace(0, len(idx) - 1, NVODE).round().astype(int)
        y0 = np.hstack([rY[sel], T[sel, None]])
        zero = np.zeros(mech.ns)
        yT = np.array([vode_cell(om, y0[c], zero, 0.0, cfg.dt) for c in range(NVODE)])
        out[f"{cfgname}/vode_sel"] = sel
        out[f"{cfgname}/vode_yT"] = yT
        out[f"{cfgname}/dt"] = np.array(cfg.dt)
        out[f"{cfgname}/rE"] = rE
        print(cfgname, "T", T[sel].round(1), "->", yT[:, -1].round(1))
    np.savez_compressed(os.path.join(HERE, "flame_states.npz"), **out)


if __name__ == "__main__":
    main()
