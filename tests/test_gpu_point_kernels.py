"""GPU parity of the pointwise kernels against the oracle: instantaneous production rates
(reactionRateRhoY, Source/PeleLM_K.H:54-98) and T from (rho h, Y) (getTfromHY,
Source/PeleLM_K.H:508-529), both in the MKS units PeleLM calls them with."""
import numpy as np
import pytest

from pelelm_gb300.reactor import reaction_rates, rhoh_to_temp
from pelelm_gb300.workloads import CONFIGS, load_mechanism, make_cells, mech_path


def _box_tensors(torch, cs, nx, ny, nz):
    n = nx * ny * nz
    ns = cs.rY.shape[1]
    rY = torch.tensor(np.ascontiguousarray(cs.rY.T.reshape(ns, nz, ny, nx) * 1e3), device="cuda")  # g/cm^3 -> kg/m^3
    rE = torch.tensor(np.ascontiguousarray(cs.rE.reshape(1, nz, ny, nx) * 0.1), device="cuda")     # erg/cm^3 -> J/m^3
    T = torch.tensor(np.ascontiguousarray(cs.T.reshape(1, nz, ny, nx)), device="cuda")
    return rY, rE, T


@pytest.mark.gpu
@pytest.mark.parametrize("mech", ["lidryer_syn", "drm19_syn"])
def test_reaction_rates_match_oracle(native_lib, oracle_mod, cuda, mech):
    torch = cuda
    cfg = CONFIGS["lidryer_amr120"] if mech == "lidryer_syn" else CONFIGS["drm19_2M"]
    nx, ny, nz = 16, 8, 4
    cs = make_cells(cfg, nx * ny * nz, seed=21)
    m = load_mechanism(mech)
    W = np.array([s.W for s in m.species])
    rY, rE, T = _box_tensors(torch, cs, nx, ny, nz)
    T_guess = T + 25.0  # the kernel refines T from (h, Y) as the reference does
    out = torch.zeros_like(rY)
    box = ((0, 0, 0), (nx - 1, ny - 1, nz - 1))
    reaction_rates(mech, box, rY, rE, T_guess, None, out)
    torch.cuda.synchronize()
    g = out.cpu().numpy().reshape(m.ns, -1).T
    om = oracle_mod.OracleMech(mech_path(mech))
    wd = om.wdot(cs.T, cs.rY / W)              # mol/cm^3/s at the true T
    ref = wd * W * 1000.0                      # kg/m^3/s
    scale = np.abs(ref).max(axis=1, keepdims=True)
    err = np.abs(g - ref) / (np.abs(ref) + 1e-9 * scale)
    assert err.max() < 1e-8, err.max()


@pytest.mark.gpu
def test_rhoh_to_temp_roundtrip(native_lib, cuda):
    torch = cuda
    cfg = CONFIGS["lidryer_amr120"]
    nx, ny, nz = 8, 8, 8
    cs = make_cells(cfg, nx * ny * nz, seed=22)
    rY, rE, T = _box_tensors(torch, cs, nx, ny, nz)
    Tg = (T * 0 + 1500.0).contiguous()
    box = ((0, 0, 0), (nx - 1, ny - 1, nz - 1))
    rhoh_to_temp("lidryer_syn", box, rY, rE, Tg, 200.0, 4000.0)
    torch.cuda.synchronize()
    np.testing.assert_allclose(Tg.cpu().numpy().reshape(-1), cs.T, rtol=1e-9)


@pytest.mark.gpu
@pytest.mark.parametrize("mech", ["lidryer_syn", "drm19_syn", "gri_syn"])
def test_heat_release_matches_numpy(native_lib, cuda, mech):
    """HeatRelease derive: -sum_k rhoYdot_k h_k(T) in W/m^3 (h_k in J/kg)."""
    import numpy as np
    from pelelm_gb300.reactor import heat_release
    from pelelm_gb300.workloads import load_mechanism, species_h_mass
    torch = cuda
    m = load_mechanism(mech)
    rng = np.random.default_rng(4)
    nx, ny, nz = 9, 5, 3
    T = rng.uniform(300.0, 2800.0, (nz, ny, nx))
    wdot = rng.normal(0.0, 50.0, (m.ns, nz, ny, nx))
    ref = -np.einsum("kzyx,zyxk->zyx", wdot, species_h_mass(m, T.reshape(-1)).reshape(nz, ny, nx, m.ns) * 1e-4)
    Tt = torch.tensor(T[None], device="cuda")
    wt = torch.tensor(wdot, device="cuda")
    out = torch.zeros(1, nz, ny, nx, dtype=torch.float64, device="cuda")
    lo = (2, -1, 7)
    heat_release(mech, (lo, (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)), Tt, wt, out)
    torch.cuda.synchronize()
    np.testing.assert_allclose(out[0].cpu().numpy(), ref, rtol=1e-11, atol=1e-9 * np.abs(ref).max())
