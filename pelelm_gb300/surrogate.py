"""Learned chemistry surrogate: an MLP that predicts a cell's (dY, dT) over dt_react.

Inputs (per cell): log10 mass fractions, T, species forcing per unit mass F_k / rho and energy
forcing F_h / rho, each normalised by training-set mean/std; outputs: dY_k and dT, normalised by
their training-set std. Hidden layers of width 256 with GELU (4 by default), BF16 weights and
activations, FP32 accumulation and FP32 master weights trained with Adam.

Every matrix product, activation, gradient and optimiser step runs in this library's own CUDA
kernels (csrc/mlp.cu: mma.sync BF16 tensor-core GEMM with fused bias/GELU epilogues, transposes,
GELU backward, MSE gradient, bias gradient, Adam); torch only holds device buffers. Training data
come from this library's own GPU BDF (the plain method) on seeded states of the benchmark
distribution.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib
from ._lib import check, lib


def _ptr(t) -> Optional[int]:
    return None if t is None else t.data_ptr()


def _pad(n: int, m: int) -> int:
    return (n + m - 1) // m * m


@dataclass
class Normalizer:
    x_mean: np.ndarray
    x_std: np.ndarray
    y_std: np.ndarray
    x_min: np.ndarray   # per-feature range seen in training (normalised units), for OOD checks
    x_max: np.ndarray


class SurrogateMLP:
    """MLP n_in -> width x depth (GELU) -> n_out with padded BF16 GEMMs on the GPU."""

    def __init__(self, torch, n_in: int, n_out: int, width: int = 256, depth: int = 4, seed: int = 0,
                 split_input: bool = True):
        self.torch = torch
        self.n_in, self.n_out, self.width, self.depth = n_in, n_out, width, depth
        # split_input: each feature enters as a (high, low) BF16 pair sharing one weight, so the
        # first layer sees ~16 significant bits of the input (BF16 alone resolves T to ~4 K).
        self.split = split_input
        self.k_half = _pad(n_in, 16) if split_input else _pad(n_in, 32)
        self.k_in = _pad(2 * self.k_half, 32) if split_input else self.k_half
        self.n_out_pad = _pad(n_out, 32)
        dims = [self.k_in] + [width] * depth + [self.n_out_pad]
        self.dims = dims
        g = torch.Generator().manual_seed(seed)
        self.W, self.b, self.Wb = [], [], []
        self.mW, self.vW, self.mb, self.vb = [], [], [], []
        for li in range(len(dims) - 1):
            fan_in = self.k_half if li == 0 else dims[li]
            fan_out = dims[li + 1]
            valid_in = n_in if li == 0 else fan_in
            valid_out = n_out if li == len(dims) - 2 else fan_out
            w = torch.zeros(fan_out, fan_in, dtype=torch.float32)
            w[:valid_out, :valid_in] = torch.randn(valid_out, valid_in, generator=g) * (2.0 / valid_in) ** 0.5
            if li == len(dims) - 2:
                w *= 0.1
            w = w.cuda()
            self.W.append(w)
            self.b.append(torch.zeros(fan_out, dtype=torch.float32, device="cuda"))
            self.Wb.append(w.to(torch.bfloat16))
            for lst in (self.mW, self.vW):
                lst.append(torch.zeros_like(w))
            for lst in (self.mb, self.vb):
                lst.append(torch.zeros(fan_out, dtype=torch.float32, device="cuda"))
        if self.split:
            self.Wb[0] = torch.zeros(dims[1], self.k_in, dtype=torch.bfloat16, device="cuda")
            self._refresh_first_layer()
        self.step_count = 0
        self.norm: Optional[Normalizer] = None

    def _refresh_first_layer(self):
        check(lib().pgb_mlp_dup_weight_bf16(_ptr(self.W[0]), self.dims[1], self.k_half, _ptr(self.Wb[0]),
                                            self.k_in, None), "dup_weight")

    def prepare_input(self, x):
        """(B, n_in) FP32 normalised features -> (B, k_in) BF16 network input."""
        torch = self.torch
        x = x.float().contiguous()
        B = x.shape[0]
        X = torch.zeros(B, self.k_in, dtype=torch.bfloat16, device="cuda")
        if self.split:
            check(lib().pgb_mlp_split_rows_bf16(_ptr(x), B, self.n_in, x.stride(0), _ptr(X), self.k_in,
                                                self.k_half, None), "split_rows")
        else:
            X[:, :self.n_in] = x.to(torch.bfloat16)
        return X

    # ------------------------------------------------------------------ kernels
    def _gemm(self, A, B, M, N, K, bias=None, act=0, pre=None, out_bf16=None, out_f32=None, ldo=None,
              n_valid=None, stream=None):
        check(lib().pgb_mlp_gemm_nt(_ptr(A), A.stride(0), _ptr(B), B.stride(0), M, N, K, _ptr(bias), act,
                                    _ptr(pre), _ptr(out_bf16), _ptr(out_f32), ldo or N,
                                    N if n_valid is None else n_valid, stream), "gemm_nt")

    def _t(self, X, rows, cols):
        out = self.torch.empty(cols, rows, dtype=self.torch.bfloat16, device="cuda")
        check(lib().pgb_mlp_transpose_bf16(_ptr(X), rows, cols, X.stride(0), _ptr(out), rows, None),
              "transpose")
        return out

    # ------------------------------------------------------------------ forward / backward
    def forward(self, X, keep=False):
        """X: (B, k_in) bf16 -> (B, n_out_pad) fp32 (normalised outputs)."""
        torch = self.torch
        B = X.shape[0]
        acts, pres = [X], []
        h = X
        for li in range(self.depth):
            N = self.dims[li + 1]
            pre = torch.empty(B, N, dtype=torch.float32, device="cuda") if keep else None
            out = torch.empty(B, N, dtype=torch.bfloat16, device="cuda")
            self._gemm(h, self.Wb[li], B, N, self.dims[li], bias=self.b[li], act=1, pre=pre, out_bf16=out)
            acts.append(out)
            pres.append(pre)
            h = out
        Y = torch.empty(B, self.n_out_pad, dtype=torch.float32, device="cuda")
        self._gemm(h, self.Wb[-1], B, self.n_out_pad, self.dims[-2], bias=self.b[-1], out_f32=Y,
                   n_valid=self.n_out)
        if keep:
            self._acts, self._pres = acts, pres
        return Y

    def backward(self, dYf, dY):
        """Gradients of the loss w.r.t. every W and b, from dL/dY (fp32 and bf16 copies)."""
        torch = self.torch
        acts, pres = self._acts, self._pres
        B = dY.shape[0]
        gW, gb = [None] * len(self.W), [None] * len(self.W)
        d_f32, d_bf = dYf, dY
        for li in range(len(self.W) - 1, -1, -1):
            N, K = self.dims[li + 1], self.dims[li]
            gb_l = torch.empty(N, dtype=torch.float32, device="cuda")
            check(lib().pgb_mlp_bias_grad(_ptr(d_f32), B, N, N, _ptr(gb_l), None), "bias_grad")
            # layer 0 of a split input: dL/dW = dZ^T x, with x ~ its high half (the gradient does
            # not need the extra bits)
            Kw = self.k_half if (li == 0 and self.split) else K
            gW_l = torch.empty(N, Kw, dtype=torch.float32, device="cuda")
            dT = self._t(d_bf, B, N)             # (N, B)
            XT = self._t(acts[li], B, Kw)        # (Kw, B)
            self._gemm(dT, XT, N, Kw, B, out_f32=gW_l)
            gW[li], gb[li] = gW_l, gb_l
            if li == 0:
                break
            WT = self._t(self.Wb[li], N, K)      # (K, N)
            dA = torch.empty(B, K, dtype=torch.float32, device="cuda")
            self._gemm(d_bf, WT, B, K, N, out_f32=dA)
            d_bf = torch.empty(B, K, dtype=torch.bfloat16, device="cuda")
            d_f32 = torch.empty(B, K, dtype=torch.float32, device="cuda")
            check(lib().pgb_mlp_gelu_backward(_ptr(dA), _ptr(pres[li - 1]), _ptr(d_bf), _ptr(d_f32),
                                              B * K, None), "gelu_backward")
        return gW, gb

    def loss_grad(self, Y, T):
        torch = self.torch
        B = Y.shape[0]
        dYf = torch.empty_like(Y)
        dY = torch.empty(Y.shape, dtype=torch.bfloat16, device="cuda")
        loss = torch.zeros(1, dtype=torch.float32, device="cuda")
        check(lib().pgb_mlp_mse_grad(_ptr(Y), _ptr(T), B, self.n_out_pad, self.n_out, _ptr(dYf), _ptr(dY),
                                     _ptr(loss), None), "mse_grad")
        return dYf, dY, loss

    def adam(self, gW, gb, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
        self.step_count += 1
        for li in range(len(self.W)):
            wb = None if (li == 0 and self.split) else self.Wb[li]
            check(lib().pgb_mlp_adam(_ptr(self.W[li]), _ptr(gW[li]), _ptr(self.mW[li]), _ptr(self.vW[li]),
                                     _ptr(wb), self.W[li].numel(), lr, b1, b2, eps, self.step_count,
                                     None), "adam")
            check(lib().pgb_mlp_adam(_ptr(self.b[li]), _ptr(gb[li]), _ptr(self.mb[li]), _ptr(self.vb[li]),
                                     None, self.b[li].numel(), lr, b1, b2, eps, self.step_count, None), "adam")
        if self.split:
            self._refresh_first_layer()

    def train_step(self, X, T, lr=1e-3) -> float:
        Y = self.forward(X, keep=True)
        dYf, dY, loss = self.loss_grad(Y, T)
        gW, gb = self.backward(dYf, dY)
        self.adam(gW, gb, lr=lr)
        return loss

    def state_dict(self):
        return {"W": [w.cpu() for w in self.W], "b": [b.cpu() for b in self.b], "dims": self.dims,
                "n_in": self.n_in, "n_out": self.n_out, "split": self.split, "norm": self.norm}


# ---------------------------------------------------------------------- features and data
def features(torch, rY, T, F, Fh, norm: Optional[Normalizer] = None, k_in: Optional[int] = None):
    """Raw (cell-major) state -> feature matrix (fp32, unnormalised unless norm given)."""
    rho = rY.sum(dim=1, keepdim=True)
    Y = rY / rho
    x = torch.cat([torch.log10(torch.clamp(Y, min=1e-14)), T[:, None], F / rho, Fh[:, None] / rho], dim=1)
    if norm is not None:
        x = (x - torch.as_tensor(norm.x_mean, device=x.device)) / torch.as_tensor(norm.x_std, device=x.device)
    if k_in is not None and x.shape[1] < k_in:
        x = torch.nn.functional.pad(x, (0, k_in - x.shape[1]))
    return x


def targets(torch, rY0, T0, rY1, T1):
    Y0 = rY0 / rY0.sum(dim=1, keepdim=True)
    Y1 = rY1 / rY1.sum(dim=1, keepdim=True)
    return torch.cat([Y1 - Y0, (T1 - T0)[:, None]], dim=1)


def fit_normalizer(x: np.ndarray, y: np.ndarray) -> Normalizer:
    xm, xs = x.mean(0), x.std(0) + 1e-12
    ys = y.std(0) + 1e-30
    z = (x - xm) / xs
    return Normalizer(x_mean=xm, x_std=xs, y_std=ys, x_min=z.min(0), x_max=z.max(0))


def surrogate_features(torch, mechanism: str, boxes) -> "torch.Tensor":
    """Raw FP32 surrogate features [cell][2 NS + 2] of the boxes' current state, computed by the
    fused inference kernel's own device code (pgb_surrogate_features)."""
    from ._lib import BoxView
    n = sum(int(b.T.numel()) for b in boxes)
    ns = int(boxes[0].rY.shape[0])
    out = torch.empty(n, 2 * ns + 2, dtype=torch.float32, device="cuda")
    arr = (BoxView * len(boxes))(*[b.view() for b in boxes])
    check(lib().pgb_surrogate_features(mechanism.encode(), arr, len(boxes), _ptr(out), None), "surrogate_features")
    return out


def generate_bdf_data(torch, cfg, ncell: int, seed: int, options: str = "gb.precision=mixed",
                      chunk: int = 1 << 20):
    """(state, forcing) -> (state after dt_react, RHS evaluations, features of the initial
    state) from this library's GPU BDF."""
    from .reactor import BoxArrays, ReactorBase
    from .workloads import make_cells
    cs = make_cells(cfg, ncell, seed=seed)
    ns = cs.rY.shape[1]
    r = ReactorBase.create("ReactorCvode", cfg.mech, f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} " + options)
    r.init(2, 1)
    outs_rY, outs_T, outs_FC, outs_x = [], [], [], []
    for c0 in range(0, ncell, chunk):
        c1 = min(ncell, c0 + chunk)
        n = c1 - c0

        def dev(a, nc):
            return torch.tensor(np.ascontiguousarray(np.asarray(a[c0:c1]).reshape(n, nc).T), device="cuda")

        rY = dev(cs.rY, ns).view(ns, 1, 1, n)
        box = BoxArrays(((0, 0, 0), (n - 1, 0, 0)), rY, dev(cs.rYsrc, ns).view(ns, 1, 1, n),
                        dev(cs.T, 1).view(1, 1, 1, n), dev(cs.rE, 1).view(1, 1, 1, n),
                        dev(cs.rEsrc, 1).view(1, 1, 1, n), torch.zeros(1, 1, 1, n, dtype=torch.float64, device="cuda"))
        outs_x.append(surrogate_features(torch, cfg.mech, [box]))
        r.react_boxes([box], cfg.dt, 0.0)
        torch.cuda.synchronize()
        outs_rY.append(box.rY.view(ns, n).T.contiguous())
        outs_T.append(box.T.view(n).clone())
        outs_FC.append(box.FC.view(n).clone())
    r.close()
    return cs, torch.cat(outs_rY), torch.cat(outs_T), torch.cat(outs_FC), torch.cat(outs_x)


# ---------------------------------------------------------------------- trained-file reader
def read_pgbs(path: str) -> dict:
    """Parses a surrogate file (layout in csrc/surrogate_io.cu) into numpy arrays."""
    import struct
    b = open(path, "rb").read()
    if b[:8] != b"PGBSURR1":
        raise ValueError(f"{path}: not a surrogate file")
    mech = b[8:40].rstrip(b"\0").decode()
    hdr = struct.unpack("<16i", b[40:104])
    ns, nmodel, nlayer, n_in, k_half, k_in, n_out, n_out_pad, nel, split = hdr[:10]
    off = [104]

    def arr(dt, n):
        a = np.frombuffer(b, dtype=dt, count=n, offset=off[0])
        off[0] += a.nbytes
        return a.copy()

    d = dict(mech=mech, ns=ns, nmodel=nmodel, nlayer=nlayer, n_in=n_in, k_half=k_half, k_in=k_in, n_out=n_out,
             n_out_pad=n_out_pad, nel=nel, split=bool(split))
    d["dims"] = arr("<i4", nlayer + 1)
    d["out_species"] = arr("<i4", n_out)
    for k in ("x_mean", "x_std", "z_min", "z_max"):
        d[k] = arr("<f8", n_in)
    d["y_scale"] = arr("<f8", n_out)
    d["A"] = arr("<f8", nel * ns).reshape(nel, ns)
    d["P"] = arr("<f8", ns * nel).reshape(ns, nel)
    g = arr("<f8", 16)
    d["gates"] = dict(zip(("ood_margin", "mis", "cons", "disT", "disY", "neg", "tol_T", "tol_Y", "audit"), g[:9]))
    d["W"], d["b"] = [], []
    for _ in range(nmodel):
        Ws, bs = [], []
        for l in range(nlayer):
            N = int(d["dims"][l + 1])
            K = k_half if (l == 0 and split) else int(d["dims"][l])
            Ws.append(arr("<f4", N * K).reshape(N, K))
            bs.append(arr("<f4", N))
        d["W"].append(Ws)
        d["b"].append(bs)
    if off[0] != len(b):
        raise ValueError(f"{path}: {len(b) - off[0]} trailing bytes")
    return d


def models_from_pgbs(torch, d: dict) -> List["SurrogateMLP"]:
    """SurrogateMLP objects carrying a trained file's weights (for checks of the fused kernel)."""
    out = []
    for mi in range(d["nmodel"]):
        m = SurrogateMLP(torch, d["n_in"], d["n_out"], width=int(d["dims"][1]), depth=d["nlayer"] - 1,
                         split_input=d["split"])
        for l in range(d["nlayer"]):
            m.W[l].copy_(torch.tensor(d["W"][mi][l]))
            m.b[l].copy_(torch.tensor(d["b"][mi][l]))
            if l > 0 or not m.split:
                m.Wb[l].copy_(m.W[l].to(torch.bfloat16))
        if m.split:
            m._refresh_first_layer()
        out.append(m)
    return out
