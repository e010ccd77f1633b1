"""Generates tests/golden/vode_cells.npz: reactor advances computed by scipy's VODE BDF.

The reference ships no golden vectors for its reactor (its CVODE-based PelePhysics reactor and
mechanisms are absent from the reference tree), so the oracle's integrator is pinned against an
independent, compiled BDF implementation: scipy.integrate.ode('vode', method='bdf'), the
Fortran ancestor of CVODE, run at rtol 1e-12 on the oracle's own right-hand side and analytic
Jacobian. The right-hand side itself is pinned separately by conservation, closed-form and
finite-difference tests.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np
from scipy.integrate import ode

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle as O  # noqa: E402
from pelelm_gb300.workloads import CONFIGS, make_cells, mech_path  # noqa: E402


def vode_cell(om, y0, F, Fh, dt, rtol=1e-12, atol=1e-20):
    def f(t, y):
        return om.rhs(y[None], F[None], np.array([Fh]))[0]

    def jac(t, y):
        return om.jac(y, F, Fh)

    r = ode(f, jac).set_integrator("vode", method="bdf", order=5, rtol=rtol, atol=atol,
                                   nsteps=1000000, with_jacobian=True)
    r.set_initial_value(y0, 0.0)
    y = r.integrate(dt)
    if not r.successful():
        raise RuntimeError("vode failed")
    return y


def main():
    out = {}
    for cfgname, n, seed in (("lidryer_32cube", 12, 101), ("lidryer_amr120", 12, 102),
                             ("drm19_2M", 6, 103), ("gri_1M", 4, 104)):
        cfg = CONFIGS[cfgname]
        om = O.OracleMech(mech_path(cfg.mech))
        cs = make_cells(cfg, n, seed=seed)
        y0 = np.hstack([cs.rY, cs.T[:, None]])
        yT = np.array([vode_cell(om, y0[c], cs.rYsrc[c], cs.rEsrc[c], cfg.dt) for c in range(n)])
        out[f"{cfgname}/y0"] = y0
        out[f"{cfgname}/F"] = cs.rYsrc
        out[f"{cfgname}/Fh"] = cs.rEsrc
        out[f"{cfgname}/yT"] = yT
        out[f"{cfgname}/dt"] = np.array(cfg.dt)
        print(cfgname, "T0", cs.T.round(1), "->", yT[:, -1].round(1))
    np.savez_compressed(os.path.join(HERE, "vode_cells.npz"), **out)


if __name__ == "__main__":
    main()
