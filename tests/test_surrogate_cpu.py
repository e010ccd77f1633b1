"""CPU tests of the surrogate's host side: mechanism-derived tables, file format round trip,
and the committed trained file's header."""
import os

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SURR = os.path.join(ROOT, "pelelm_gb300", "data", "drm19_syn.pgbs")


def test_active_species_and_element_projection():
    from pelelm_gb300.surrogate_train import active_species, element_projection
    from pelelm_gb300.workloads import load_mechanism
    mech = load_mechanism("drm19_syn")
    act = active_species(mech)
    names = [mech.species[k].name for k in act]
    assert "N2" not in names and "AR" not in names      # inert in this mechanism
    assert {"CH4", "O2", "H2O", "CO2", "OH", "H"} <= set(names)
    A, P = element_projection(mech, act)
    assert A.shape == (3, mech.ns) and P.shape == (mech.ns, 3)  # C, H, O
    rng = np.random.default_rng(0)
    dY = np.zeros((50, mech.ns))
    dY[:, act] = rng.normal(size=(50, len(act))) * 1e-3
    corr = -(dY @ A.T) @ P.T
    assert np.abs((dY + corr) @ A.T).max() <= 1e-14 * np.abs(dY @ A.T).max()
    # least norm: the correction is orthogonal to the conserving subspace (lies in span A^T)
    assert np.allclose(corr @ (np.eye(mech.ns) - A.T @ np.linalg.pinv(A.T)), 0.0, atol=1e-15)
    # inert species are never corrected
    inert = [k for k in range(mech.ns) if k not in act]
    assert np.all(corr[:, inert] == 0.0)


class _FakeModel:
    def __init__(self, rng, dims, k_half, n_in):
        import torch
        self.dims, self.k_half, self.k_in, self.n_in, self.n_out_pad, self.split = dims, k_half, dims[0], n_in, dims[-1], True
        self.W = [torch.tensor(rng.normal(size=(dims[l + 1], k_half if l == 0 else dims[l])), dtype=torch.float32)
                  for l in range(len(dims) - 1)]
        self.b = [torch.tensor(rng.normal(size=dims[l + 1]), dtype=torch.float32) for l in range(len(dims) - 1)]


def test_pgbs_round_trip(tmp_path):
    pytest.importorskip("torch")
    from pelelm_gb300.surrogate import read_pgbs
    from pelelm_gb300.surrogate_train import write_pgbs
    rng = np.random.default_rng(3)
    ns, n_in = 21, 44
    dims = [96, 256, 256, 32]
    models = [_FakeModel(rng, dims, 48, n_in) for _ in range(2)]
    A = rng.normal(size=(3, ns))
    P = rng.normal(size=(ns, 3))
    osp = list(range(19)) + [-1]
    gates = dict(ood_margin=0.05, mis=0.3, cons=1e-5, disT=0.3, disY=1e-5, neg=1e-6, tol_T=1.0, tol_Y=1e-4,
                 audit=0.01)
    arrs = [rng.normal(size=n_in) for _ in range(4)]
    ys = rng.uniform(1e-3, 1.0, size=len(osp))
    path = tmp_path / "t.pgbs"
    write_pgbs(str(path), "drm19_syn", ns, models, *arrs, ys, osp, A, P, gates)
    d = read_pgbs(str(path))
    assert d["mech"] == "drm19_syn" and d["ns"] == ns and d["nmodel"] == 2 and d["nlayer"] == 3
    assert d["k_half"] == 48 and d["k_in"] == 96 and d["split"]
    assert list(d["dims"]) == dims and list(d["out_species"]) == osp
    for k, a in zip(("x_mean", "x_std", "z_min", "z_max"), arrs):
        np.testing.assert_array_equal(d[k], a)
    np.testing.assert_array_equal(d["y_scale"], ys)
    np.testing.assert_array_equal(d["A"], A)
    np.testing.assert_array_equal(d["P"], P)
    assert d["gates"]["mis"] == 0.3 and d["gates"]["audit"] == 0.01
    for m, Ws, bs in zip(models, d["W"], d["b"]):
        for W, b, Wr, br in zip(m.W, m.b, Ws, bs):
            np.testing.assert_array_equal(W.numpy(), Wr)
            np.testing.assert_array_equal(b.numpy(), br)


def test_committed_surrogate_file_matches_drm19():
    from pelelm_gb300.surrogate import read_pgbs
    from pelelm_gb300.workloads import load_mechanism
    d = read_pgbs(SURR)
    mech = load_mechanism("drm19_syn")
    assert d["mech"] == "drm19_syn" and d["ns"] == mech.ns and d["n_in"] == 2 * mech.ns + 2
    assert d["nlayer"] == 5 and list(d["dims"][1:-1]) == [256] * 4   # 4 hidden layers of 256
    assert d["out_species"][-1] == -1 and d["n_out"] == len(d["out_species"])
    assert d["gates"]["tol_T"] == 1.0 and d["gates"]["tol_Y"] == 1e-4 and d["gates"]["audit"] == 0.01
    assert np.all(d["x_std"] > 0)
