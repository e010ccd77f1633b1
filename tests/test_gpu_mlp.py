"""Tensor-core kernels of the surrogate: the BF16 GEMM against a plain PyTorch FP32 reference,
and the full training step's gradients against the FP64 CPU reference (oracle/mlp_oracle.py)."""
import numpy as np
import pytest

from pelelm_gb300 import _lib


@pytest.mark.gpu
@pytest.mark.parametrize("M,N,K", [(256, 256, 64), (300, 40, 256), (8192, 32, 256), (64, 256, 32)])
@pytest.mark.parametrize("act", [0, 1])
def test_gemm_nt_matches_fp32_reference(native_lib, cuda, M, N, K, act):
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(M + N + K)
    A = torch.randn(M, K, device="cuda", generator=g).to(torch.bfloat16)
    B = torch.randn(N, K, device="cuda", generator=g).to(torch.bfloat16)
    bias = torch.randn(N, device="cuda", generator=g)
    out = torch.empty(M, N, dtype=torch.float32, device="cuda")
    pre = torch.empty(M, N, dtype=torch.float32, device="cuda")
    rc = native_lib.pgb_mlp_gemm_nt(A.data_ptr(), K, B.data_ptr(), K, M, N, K, bias.data_ptr(), act,
                                    pre.data_ptr(), None, out.data_ptr(), N, N, None)
    assert rc == 0, _lib.last_error()
    ref = A.float() @ B.float().T + bias
    torch.testing.assert_close(pre, ref, rtol=1e-4, atol=1e-3)
    if act:
        ref = torch.nn.functional.gelu(ref, approximate="tanh")
    torch.testing.assert_close(out, ref, rtol=1e-4, atol=1e-3)


@pytest.mark.gpu
def test_training_gradients_match_fp64_reference(native_lib, cuda):
    import mlp_oracle
    from pelelm_gb300.surrogate import SurrogateMLP
    torch = cuda
    B, n_in, n_out = 512, 44, 22
    m = SurrogateMLP(torch, n_in, n_out, width=64, depth=3, seed=3)
    rng = np.random.default_rng(0)
    X = np.zeros((B, m.k_in), dtype=np.float32)
    X[:, :n_in] = rng.normal(size=(B, n_in))
    T = np.zeros((B, m.n_out_pad), dtype=np.float32)
    T[:, :n_out] = rng.normal(size=(B, n_out))
    Xg = torch.tensor(X, device="cuda").to(torch.bfloat16)
    Tg = torch.tensor(T, device="cuda")
    Y = m.forward(Xg, keep=True)
    dYf, dY, loss = m.loss_grad(Y, Tg)
    gW, gb = m.backward(dYf, dY)
    Ws = [w.to(torch.bfloat16).double().cpu().numpy() for w in m.W]
    bs = [b.double().cpu().numpy() for b in m.b]
    Xr = Xg.double().cpu().numpy()
    loss_ref, gW_ref, gb_ref = mlp_oracle.loss_and_grads(Ws, bs, Xr, T.astype(np.float64), n_out)
    assert abs(float(loss) - loss_ref) <= 0.02 * loss_ref
    for li in range(len(Ws)):
        a = gW[li].double().cpu().numpy().ravel()
        r = gW_ref[li].ravel()
        cos = a @ r / (np.linalg.norm(a) * np.linalg.norm(r) + 1e-300)
        assert cos > 0.999, (li, cos)
        assert np.linalg.norm(a - r) <= 0.03 * np.linalg.norm(r), li
        np.testing.assert_allclose(gb[li].double().cpu().numpy(), gb_ref[li], rtol=0.05,
                                   atol=0.03 * np.abs(gb_ref[li]).max())


@pytest.mark.gpu
def test_adam_training_reduces_loss(native_lib, cuda):
    from pelelm_gb300.surrogate import SurrogateMLP
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(1)
    n_in, n_out, B = 20, 10, 2048
    m = SurrogateMLP(torch, n_in, n_out, width=128, depth=3, seed=1)
    X = torch.zeros(B, m.k_in, device="cuda")
    X[:, :n_in] = torch.randn(B, n_in, device="cuda", generator=g)
    T = torch.zeros(B, m.n_out_pad, device="cuda")
    T[:, :n_out] = torch.sin(X[:, :n_out]) * torch.cos(X[:, n_out:2 * n_out])
    Xb = X.to(torch.bfloat16)
    losses = [float(m.train_step(Xb, T, lr=2e-3)) for _ in range(200)]
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
