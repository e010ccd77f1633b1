"""ctypes wrapper of the CPU oracle (liboracle.so). TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py use this
module. Parity against the reference is UNPINNED (its reactor, mechanisms and CVODE are
absent from the reference tree and it ships no golden vectors); the oracle is pinned by
closed-form known-answer tests and scipy VODE cross-checks instead.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "liboracle.so")

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
_lp = C.POINTER(C.c_long)


def build(force: bool = False) -> str:
    """make (incremental: rebuilds when a source is newer than the library)."""
    subprocess.check_call(["make", "-s", "-C", HERE] + (["-B"] if force else []))
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB_PATH)
        L.orc_mech_load.restype = C.c_void_p
        L.orc_mech_load.argtypes = [C.c_char_p]
        L.orc_mech_free.argtypes = [C.c_void_p]
        L.orc_mech_ns.argtypes = [C.c_void_p]
        L.orc_mech_nr.argtypes = [C.c_void_p]
        L.orc_wdot_cells.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.orc_rhs_cells.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp]
        L.orc_jac.argtypes = [C.c_void_p, _dp, _dp, C.c_double, _dp]
        L.orc_count_rhs.argtypes = [C.c_void_p, _dp, _dp, C.c_double, _lp, _lp]
        L.orc_mixture_h.restype = C.c_double
        L.orc_mixture_h.argtypes = [C.c_void_p, C.c_double, _dp]
        L.orc_hy2t_cells.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp]
        L.orc_react_cells.restype = C.c_int
        L.orc_react_cells.argtypes = [C.c_void_p, C.c_int, _dp, _dp, _dp, _dp, _dp, _dp, _ip,
                                      C.c_double, C.c_double, _dp, C.c_int, C.c_int, C.c_int, _lp]
        L.orc_bdf_one.restype = C.c_int
        L.orc_bdf_one.argtypes = [C.c_void_p, _dp, _dp, C.c_double, C.c_double, C.c_double, _dp,
                                  C.c_int, C.c_int, _lp]
        L.orc_max_threads.restype = C.c_int
        L.orc_lu_solve.restype = C.c_int
        L.orc_lu_solve.argtypes = [C.c_int, _dp, _dp, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


class OracleMech:
    def __init__(self, path: str):
        self.path = path
        self.h = lib().orc_mech_load(path.encode())
        if not self.h:
            raise RuntimeError(f"oracle: failed to load mechanism {path}")
        self.ns = lib().orc_mech_ns(self.h)
        self.nr = lib().orc_mech_nr(self.h)

    def __del__(self):
        try:
            if self.h:
                lib().orc_mech_free(self.h)
        except Exception:
            pass

    def wdot(self, T, Cc):
        T = np.ascontiguousarray(T, dtype=np.float64)
        Cc = np.ascontiguousarray(Cc, dtype=np.float64).reshape(T.size, self.ns)
        out = np.empty_like(Cc)
        lib().orc_wdot_cells(self.h, T.size, _d(T), _d(Cc), _d(out))
        return out

    def rhs(self, y, F, Fh):
        y = np.ascontiguousarray(y, dtype=np.float64).reshape(-1, self.ns + 1)
        n = y.shape[0]
        F = np.ascontiguousarray(F, dtype=np.float64).reshape(n, self.ns)
        Fh = np.ascontiguousarray(Fh, dtype=np.float64).reshape(n)
        out = np.empty_like(y)
        lib().orc_rhs_cells(self.h, n, _d(y), _d(F), _d(Fh), _d(out))
        return out

    def jac(self, y, F, Fh):
        y = np.ascontiguousarray(y, dtype=np.float64)
        F = np.ascontiguousarray(F, dtype=np.float64)
        J = np.empty((self.ns + 1, self.ns + 1))
        lib().orc_jac(self.h, _d(y), _d(F), float(Fh), _d(J))
        return J

    def count_rhs(self, y, F, Fh):
        y = np.ascontiguousarray(y, dtype=np.float64)
        F = np.ascontiguousarray(F, dtype=np.float64)
        ops, trans = C.c_long(), C.c_long()
        lib().orc_count_rhs(self.h, _d(y), _d(F), float(Fh), C.byref(ops), C.byref(trans))
        return ops.value, trans.value

    def mixture_h(self, T, Y):
        Y = np.ascontiguousarray(Y, dtype=np.float64)
        return lib().orc_mixture_h(self.h, float(T), _d(Y))

    def hy2t(self, h, Y, Tguess):
        h = np.ascontiguousarray(h, dtype=np.float64)
        Y = np.ascontiguousarray(Y, dtype=np.float64).reshape(h.size, self.ns)
        T = np.array(Tguess, dtype=np.float64, copy=True).reshape(h.size)
        lib().orc_hy2t_cells(self.h, h.size, _d(h), _d(Y), _d(T))
        return T

    def react(self, rY, rYsrc, T, rE, rEsrc, mask, dt, rtol, atol, max_order=5,
              max_steps=20000, nthreads=0, with_stats=False):
        """Cell-major inputs (ncell, ns) etc.; returns (rY, T, rE, FC, nfail[, stats])."""
        n = T.size
        rYc = np.ascontiguousarray(np.asarray(rY, dtype=np.float64).T).copy()
        rYs = np.ascontiguousarray(np.asarray(rYsrc, dtype=np.float64).T)
        Tn = np.array(T, dtype=np.float64, copy=True)
        rEn = np.array(rE, dtype=np.float64, copy=True)
        rEs = np.ascontiguousarray(rEsrc, dtype=np.float64)
        FC = np.zeros(n)
        m = np.ascontiguousarray(mask, dtype=np.int32)
        at = np.ascontiguousarray(np.broadcast_to(np.asarray(atol, dtype=np.float64), (self.ns + 1,)))
        stats = np.zeros((n, 6), dtype=np.int64) if with_stats else None
        nfail = lib().orc_react_cells(self.h, n, _d(rYc), _d(rYs), _d(Tn), _d(rEn), _d(rEs), _d(FC),
                                      m.ctypes.data_as(_ip), float(dt), float(rtol), _d(at),
                                      int(max_order), int(max_steps), int(nthreads),
                                      stats.ctypes.data_as(_lp) if with_stats else None)
        out = (rYc.T.copy(), Tn, rEn, FC, nfail)
        return out + (stats,) if with_stats else out

    def bdf_one(self, y, F, Fh, dt, rtol, atol, max_order=5, max_steps=100000):
        y = np.array(y, dtype=np.float64, copy=True)
        F = np.ascontiguousarray(F, dtype=np.float64)
        at = np.ascontiguousarray(np.broadcast_to(np.asarray(atol, dtype=np.float64), (self.ns + 1,)))
        st = np.zeros(6, dtype=np.int64)
        status = lib().orc_bdf_one(self.h, _d(y), _d(F), float(Fh), float(dt), float(rtol), _d(at),
                                   int(max_order), int(max_steps), st.ctypes.data_as(_lp))
        return y, status, st


def max_threads() -> int:
    return lib().orc_max_threads()


def lu_solve(A, b):
    """The integrator's partial-pivot LU on one system; returns x, or None when singular."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.empty_like(b)
    return None if lib().orc_lu_solve(A.shape[0], _d(A), _d(b), _d(x)) else x
