"""The analytic Jacobian and the dense Newton solve of the warp and lane-group BDF kernels, held
directly against the oracle. Inside the reactor call at Source/PeleLM.cpp:5752 these are CVODE's
analytic Jacobian and dense direct solve (cvode.solve_type = denseAJ_direct); the kernels build
them in warp_setup (per-reaction partials, the generated contribution program, the energy row,
partial-pivot LU) and solve with warp_lu_solve. The diagnostic entry point pgb_newton_matrix runs
that production code on a batch of states:

* FP64 J against the oracle's dense analytic Jacobian (oracle/chem_oracle.cpp), entry by entry,
  relative to the largest entry of its row (the two sum the same terms in different orders);
* the FP32 Newton matrix I - gamma J of mixed precision against the FP64 one at FP32 tolerance
  (what the Newton iteration uses: rows of J far below FP32's range, where the FP32 path's
  clamped exponentials dominate, are negligible next to the identity);
* x solving (I - gamma J) x = b: normwise backward error of the GPU solution on the GPU's own
  matrix, at the working precision of each mode (FP64 LU, FP32 LU);
* the cell-per-thread kernels' Jacobian (the generated one of the 9-species mechanism, the
  table-driven one of the 21-species mechanism) against the oracle the same way.
"""
import numpy as np
import pytest

from pelelm_gb300 import _lib
from pelelm_gb300.workloads import CONFIGS, make_cells, mech_path

CASES = [("lidryer_amr120", 256), ("drm19_2M", 512), ("gri_1M", 256)]
GAMMA = 1e-7  # a BDF gamma = h l_1 of the early, small steps


def _states(cfgname, n):
    cfg = CONFIGS[cfgname]
    cs = make_cells(cfg, n, seed=99)
    y = np.concatenate([cs.rY, cs.T[:, None]], axis=1)
    b = np.random.default_rng(5).normal(size=y.shape)
    return cfg, cs, y, b


def _gpu(torch, cfg, cs, y, b, fp64, mapping=1):
    n, N = y.shape
    dev = dict(device="cuda", dtype=torch.float64)
    ty, tF = torch.tensor(y, **dev), torch.tensor(cs.rYsrc, **dev)
    tFh, tb = torch.tensor(cs.rEsrc, **dev), torch.tensor(b, **dev)
    J = torch.empty((n, N, N), **dev)
    x = torch.empty((n, N), **dev)
    rc = _lib.lib().pgb_newton_matrix(cfg.mech.encode(), mapping, n, ty.data_ptr(), tF.data_ptr(),
                                      tFh.data_ptr(), GAMMA, tb.data_ptr(), int(fp64), J.data_ptr(),
                                      x.data_ptr(), None)
    assert rc == 0, _lib.last_error()
    torch.cuda.synchronize()
    return J.cpu().numpy(), x.cpu().numpy()


def _backward_error(J, x, b):
    """max over cells of ||(I - gamma J) x - b||_inf / (||I - gamma J||_inf ||x||_inf + ||b||_inf)
    (the normwise bound a partial-pivot LU guarantees)"""
    N = J.shape[1]
    M = np.eye(N)[None] - GAMMA * J
    r = np.einsum("cij,cj->ci", M, x) - b
    den = np.abs(M).sum(axis=2).max(axis=1) * np.abs(x).max(axis=1) + np.abs(b).max(axis=1)
    return float(np.max(np.abs(r).max(axis=1) / den))


def _componentwise_error(J, x, b):
    """max over cells and rows of |r_i| / (|M| |x| + |b|)_i (reported, not asserted)"""
    N = J.shape[1]
    M = np.eye(N)[None] - GAMMA * J
    r = np.einsum("cij,cj->ci", M, x) - b
    den = np.einsum("cij,cj->ci", np.abs(M), np.abs(x)) + np.abs(b)
    return float(np.max(np.abs(r) / den))


@pytest.mark.gpu
@pytest.mark.parametrize("cfgname,n", CASES)
def test_fp64_jacobian_and_solve_match_the_oracle(native_lib, oracle_mod, cuda, cfgname, n):
    torch = cuda
    cfg, cs, y, b = _states(cfgname, n)
    Jg, xg = _gpu(torch, cfg, cs, y, b, fp64=True)
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    worst = 0.0
    for c in range(n):
        Jo = om.jac(y[c], cs.rYsrc[c], cs.rEsrc[c])
        scale = np.abs(Jo).max(axis=1, keepdims=True) + 1e-300
        worst = max(worst, float(np.max(np.abs(Jg[c] - Jo) / scale)))
    assert np.isfinite(Jg).all()
    assert worst <= 1e-9, f"{cfg.mech}: FP64 Jacobian differs from the oracle by {worst:.3e} of its row scale"
    assert np.isfinite(xg).all(), "a Newton matrix was reported singular"
    be = _backward_error(Jg, xg, b)
    assert be <= 1e-13, f"{cfg.mech}: FP64 LU solve backward error {be:.3e}"
    print(f"{cfg.mech}: FP64 J vs oracle {worst:.2e} of row scale, solve backward error {be:.2e} "
          f"(componentwise {_componentwise_error(Jg, xg, b):.2e})")


@pytest.mark.gpu
@pytest.mark.parametrize("cfgname,n", CASES)
def test_fp32_jacobian_and_solve_of_mixed_precision(native_lib, cuda, cfgname, n):
    torch = cuda
    cfg, cs, y, b = _states(cfgname, n)
    J64, _ = _gpu(torch, cfg, cs, y, b, fp64=True)
    J32, x32 = _gpu(torch, cfg, cs, y, b, fp64=False)
    assert np.isfinite(J32).all() and np.isfinite(x32).all()
    eye = np.eye(J64.shape[1])[None]
    M64, M32 = eye - GAMMA * J64, eye - GAMMA * J32
    representable = np.abs(M64).max(axis=(1, 2)) < 1e37  # FP32 can hold the FP64 matrix
    rel = (np.abs(M32 - M64) / np.abs(M64).max(axis=2, keepdims=True)).max(axis=(1, 2))
    worst = float(rel[representable].max())
    assert representable.mean() >= 0.99, f"{cfg.mech}: {np.sum(~representable)} Newton matrices beyond FP32 range"
    assert worst <= 1e-4, f"{cfg.mech}: FP32 Newton matrix differs from FP64 by {worst:.3e} of its row scale"
    be = _backward_error(J32, x32, b)
    assert be <= 1e-5, f"{cfg.mech}: FP32 LU solve backward error {be:.3e}"
    print(f"{cfg.mech}: FP32 I - gamma J vs FP64 {worst:.2e} of row scale (p99 "
          f"{np.quantile(rel[representable], 0.99):.2e}; {np.sum(~representable)} of {n} beyond FP32 range), "
          f"solve backward error {be:.2e} (componentwise {_componentwise_error(J32, x32, b):.2e})")


def _oracle_rel(om, y, cs, J):
    worst = 0.0
    for c in range(y.shape[0]):
        Jo = om.jac(y[c], cs.rYsrc[c], cs.rEsrc[c])
        worst = max(worst, float(np.max(np.abs(J[c] - Jo) / (np.abs(Jo).max(axis=1, keepdims=True) + 1e-300))))
    return worst


@pytest.mark.gpu
@pytest.mark.parametrize("cfgname,n", CASES[:2])
def test_per_thread_jacobian_matches_the_oracle(native_lib, oracle_mod, cuda, cfgname, n):
    torch = cuda
    cfg, cs, y, b = _states(cfgname, n)
    om = oracle_mod.OracleMech(mech_path(cfg.mech))
    J64, x = _gpu(torch, cfg, cs, y, b, fp64=True, mapping=0)
    assert np.isnan(x).all()  # the per-thread variant computes J only
    worst = _oracle_rel(om, y, cs, J64)
    assert worst <= 1e-9, f"{cfg.mech}: per-thread FP64 Jacobian differs from the oracle by {worst:.3e}"
    J32, _ = _gpu(torch, cfg, cs, y, b, fp64=False, mapping=0)
    eye = np.eye(J64.shape[1])[None]
    M64, M32 = eye - GAMMA * J64, eye - GAMMA * J32
    rel = float((np.abs(M32 - M64) / np.abs(M64).max(axis=2, keepdims=True)).max())
    assert np.isfinite(J32).all() and rel <= 1e-4, f"{cfg.mech}: per-thread FP32 Newton matrix off by {rel:.3e}"
    print(f"{cfg.mech}: per-thread FP64 J vs oracle {worst:.2e} of row scale; FP32 I - gamma J vs FP64 {rel:.2e}")


@pytest.mark.gpu
def test_per_thread_jacobian_refused_without_per_thread_kernels(native_lib, cuda):
    torch = cuda
    cfg, cs, y, b = _states("gri_1M", 32)
    with pytest.raises(AssertionError, match="cell-per-thread"):
        _gpu(torch, cfg, cs, y, b, fp64=True, mapping=0)
