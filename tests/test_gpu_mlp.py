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
    m = SurrogateMLP(torch, n_in, n_out, width=64, depth=3, seed=3, split_input=False)
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
def test_split_input_carries_16_bits_and_gradients_match(native_lib, cuda):
    """Split input: x enters as BF16 (high, low) halves sharing one first-layer weight."""
    import mlp_oracle
    from pelelm_gb300.surrogate import SurrogateMLP
    torch = cuda
    B, n_in, n_out = 512, 44, 22
    m = SurrogateMLP(torch, n_in, n_out, width=64, depth=3, seed=5, split_input=True)
    assert m.k_half == 48 and m.k_in == 96
    rng = np.random.default_rng(2)
    x = rng.normal(size=(B, n_in)).astype(np.float32)
    X = m.prepare_input(torch.tensor(x, device="cuda"))
    Xd = X.double().cpu().numpy()
    recon = Xd[:, :n_in] + Xd[:, m.k_half:m.k_half + n_in]
    assert np.abs(recon - x).max() <= 2.0 ** -15 * np.abs(x).max()
    assert np.abs(Xd[:, :n_in] - x).max() > 2.0 ** -10 * np.abs(x).max()   # BF16 alone is coarser
    # the BF16 first-layer weight is the FP32 master rounded, twice
    Wb0 = m.Wb[0].double().cpu().numpy()
    np.testing.assert_array_equal(Wb0[:, :m.k_half], Wb0[:, m.k_half:2 * m.k_half])
    np.testing.assert_array_equal(Wb0[:, :m.k_half], m.W[0].to(torch.bfloat16).double().cpu().numpy())
    T = np.zeros((B, m.n_out_pad), dtype=np.float32)
    T[:, :n_out] = rng.normal(size=(B, n_out))
    Y = m.forward(X, keep=True)
    dYf, dY, loss = m.loss_grad(Y, torch.tensor(T, device="cuda"))
    gW, gb = m.backward(dYf, dY)
    Ws = [w.to(torch.bfloat16).double().cpu().numpy() for w in m.W]
    bs = [b.double().cpu().numpy() for b in m.b]
    Xr = np.zeros((B, m.k_half))
    Xr[:, :n_in] = recon
    loss_ref, gW_ref, gb_ref = mlp_oracle.loss_and_grads(Ws, bs, Xr, T.astype(np.float64), n_out)
    assert abs(float(loss) - loss_ref) <= 0.02 * loss_ref
    for li in range(len(Ws)):
        a = gW[li].double().cpu().numpy().ravel()
        r = gW_ref[li].ravel()
        assert a.shape == r.shape
        assert np.linalg.norm(a - r) <= 0.03 * np.linalg.norm(r), li


@pytest.mark.gpu
def test_adam_training_reduces_loss(native_lib, cuda):
    from pelelm_gb300.surrogate import SurrogateMLP
    torch = cuda
    g = torch.Generator(device="cuda").manual_seed(1)
    n_in, n_out, B = 20, 10, 2048
    m = SurrogateMLP(torch, n_in, n_out, width=128, depth=3, seed=1)
    x = torch.randn(B, n_in, device="cuda", generator=g)
    T = torch.zeros(B, m.n_out_pad, device="cuda")
    T[:, :n_out] = torch.sin(x[:, :n_out]) * torch.cos(x[:, n_out:2 * n_out])
    Xb = m.prepare_input(x)
    losses = [float(m.train_step(Xb, T, lr=2e-3)) for _ in range(200)]
    assert losses[-1] < 0.2 * losses[0], (losses[0], losses[-1])
