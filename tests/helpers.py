"""Shared helpers for the parity tests: layout cells into boxes on the GPU, run the oracle."""
import numpy as np

from pelelm_gb300.reactor import BoxArrays


def boxes_from_cells(torch, cs, sides_or_shapes, lo_list=None, ghost=0, with_mask=False):
    """Split the flat cell state `cs` into boxes (each (nx,ny,nz) or cube side), one
    FArrayBox-like tensor per field with optional ghost cells around the valid box."""
    out = []
    c0 = 0
    for b, s in enumerate(sides_or_shapes):
        nx, ny, nz = (s, s, s) if np.isscalar(s) else s
        n = nx * ny * nz
        lo = (0, 0, 0) if lo_list is None else lo_list[b]
        sl = slice(c0, c0 + n)
        c0 += n

        def field(a, ncomp):
            a = np.asarray(a[sl], dtype=np.float64).reshape(n, ncomp).T.reshape(ncomp, nz, ny, nx)
            full = np.zeros((ncomp, nz + 2 * ghost, ny + 2 * ghost, nx + 2 * ghost))
            full[:, ghost:ghost + nz, ghost:ghost + ny, ghost:ghost + nx] = a
            t = torch.tensor(np.ascontiguousarray(full), device="cuda")
            return t, t[:, ghost:ghost + nz, ghost:ghost + ny, ghost:ghost + nx]

        ns = cs.rY.shape[1]
        fields = {}
        for name, arr, nc in (("rY", cs.rY, ns), ("rY_src", cs.rYsrc, ns), ("T", cs.T, 1),
                              ("rEner", cs.rE, 1), ("rEner_src", cs.rEsrc, 1),
                              ("FC", np.zeros(cs.T.size), 1)):
            fields[name] = field(arr, nc)[1]
        mask = None
        if with_mask:
            m = np.asarray(cs.mask[sl], dtype=np.int32).reshape(nz, ny, nx)
            mask = torch.tensor(np.ascontiguousarray(m[None]), device="cuda")
        hi = (lo[0] + nx - 1, lo[1] + ny - 1, lo[2] + nz - 1)
        out.append(BoxArrays((lo, hi), fields["rY"], fields["rY_src"], fields["T"], fields["rEner"],
                             fields["rEner_src"], fields["FC"], mask))
    return out


def gather(boxes, ns):
    """Back to flat cell-major numpy arrays (rY (n,ns), T, rE, FC)."""
    rY, T, rE, FC = [], [], [], []
    for b in boxes:
        nc, nz, ny, nx = b.rY.shape
        n = nx * ny * nz
        rY.append(b.rY.cpu().numpy().reshape(ns, n).T)
        T.append(b.T.cpu().numpy().reshape(n))
        rE.append(b.rEner.cpu().numpy().reshape(n))
        FC.append(b.FC.cpu().numpy().reshape(n))
    return np.vstack(rY), np.concatenate(T), np.concatenate(rE), np.concatenate(FC)


def tol_ratio(y_gpu, y_ref, rtol, atol):
    """max over entries of |dy| / (atol + rtol |y_ref|)."""
    return np.abs(y_gpu - y_ref) / (atol + rtol * np.abs(y_ref))


def outliers_within_global_error(om, cs, cells, gpu, orc, dt, rtol):
    """Cells outside the plain tolerances have taken another step sequence (a last-bit
    difference in a sum can move an adaptive BDF onto other steps). Each is held, cell by
    cell, to the oracle's own global error on that cell against a tight oracle (rtol 1e-11):
    |GPU - tight| <= 2 |oracle - tight| + 50 rtol (T relative, mass fractions absolute).
    gpu / orc: (rY, T) cell-major arrays of the same cells as `cells` indexes into cs."""
    if len(cells) == 0:
        return
    c = np.asarray(cells)
    t = om.react(cs.rY[c], cs.rYsrc[c], cs.T[c], cs.rE[c], cs.rEsrc[c], cs.mask[c], dt, 1e-11, 1e-16,
                 max_steps=200000)
    Yt = t[0] / t[0].sum(1, keepdims=True)
    (rYg, Tg), (rYo, To) = gpu, orc
    eTg, eTo = np.abs(Tg - t[1]), np.abs(To - t[1])
    eYg = np.abs(rYg / rYg.sum(1, keepdims=True) - Yt).max(1)
    eYo = np.abs(rYo / rYo.sum(1, keepdims=True) - Yt).max(1)
    assert np.all(eTg <= 2 * eTo + 50 * rtol * t[1]), (c, eTg, eTo)
    assert np.all(eYg <= 2 * eYo + 50 * rtol), (c, eYg, eYo)
