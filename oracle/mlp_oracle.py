"""FP64 CPU reference of the surrogate MLP (TEST INFRASTRUCTURE ONLY): forward pass and exact
gradients of the mean-squared error for the architecture the GPU kernels implement — dense
layers with tanh-form GELU on the hidden layers, identity output, loss averaged over the
batch and the valid outputs."""
import numpy as np

C0 = 0.7978845608028654
C1 = 0.044715


def gelu(x):
    return 0.5 * x * (1.0 + np.tanh(C0 * (x + C1 * x ** 3)))


def gelu_grad(x):
    t = np.tanh(C0 * (x + C1 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * C0 * (1.0 + 3.0 * C1 * x * x)


def forward(Ws, bs, X):
    acts, pres = [X], []
    h = X
    for W, b in zip(Ws[:-1], bs[:-1]):
        z = h @ W.T + b
        pres.append(z)
        h = gelu(z)
        acts.append(h)
    return h @ Ws[-1].T + bs[-1], acts, pres


def loss_and_grads(Ws, bs, X, T, n_valid):
    Y, acts, pres = forward(Ws, bs, X)
    B = X.shape[0]
    d = np.zeros_like(Y)
    d[:, :n_valid] = Y[:, :n_valid] - T[:, :n_valid]
    loss = float((d ** 2).sum())
    g = 2.0 * d / (B * n_valid)
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    for li in range(len(Ws) - 1, -1, -1):
        gW[li] = g.T @ acts[li]
        gb[li] = g.sum(axis=0)
        if li == 0:
            break
        g = (g @ Ws[li]) * gelu_grad(pres[li - 1])
    return loss, gW, gb
