"""Host-side mirror of the reference reactor interface for Python callers (tests, bench).

PeleLM holds a ``pele::physics::reactions::ReactorBase`` (Source/PeleLM.H:673-674) and calls
``create`` / ``init`` (Source/PeleLM.cpp:706-709), ``set_typ_vals_ode`` (:1513), ``react``
(:5752-5757) and ``close`` (:930). This module keeps those names, argument meanings and error
behaviour (``react`` returns the number of failed cells; failed cells carry FC < 0) and
forwards every call to the native library through its C ABI. Arrays are CUDA tensors laid out
like an AMReX FArrayBox: ``(ncomp, nz, ny, nx)``, i fastest.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import List, Optional, Sequence, Tuple

from . import _lib
from ._lib import Array4, BoxView, Stats, check, lib

Box = Tuple[Tuple[int, int, int], Tuple[int, int, int]]  # (lo, hi), inclusive like amrex::Box


def array4(t, lo=(0, 0, 0)) -> Array4:
    """Array4 view of a CUDA tensor shaped (ncomp, nz, ny, nx) whose first cell is at lo."""
    if t is None:
        return Array4()
    if t.dim() == 3:
        t = t.unsqueeze(0)
    if t.dim() != 4:
        raise ValueError("expected a (ncomp, nz, ny, nx) tensor")
    if not t.is_cuda:
        raise ValueError("reactor arrays must be CUDA tensors")
    st = t.stride()
    if st[3] != 1:
        raise ValueError("the i direction must be contiguous")
    a = Array4()
    a.p = t.data_ptr()
    a.jstride, a.kstride, a.nstride = st[2], st[1], st[0]
    nc, nz, ny, nx = t.shape
    a.begin = (C.c_int * 3)(lo[0], lo[1], lo[2])
    a.end = (C.c_int * 3)(lo[0] + nx, lo[1] + ny, lo[2] + nz)
    a.ncomp = nc
    return a


@dataclass
class BoxArrays:
    """The react() arguments of one box."""
    box: Box
    rY: object
    rY_src: object
    T: object
    rEner: object
    rEner_src: object
    FC: object
    mask: Optional[object] = None

    def view(self) -> BoxView:
        lo = self.box[0]
        v = BoxView()
        v.box.lo = (C.c_int * 3)(*self.box[0])
        v.box.hi = (C.c_int * 3)(*self.box[1])
        v.rY = array4(self.rY, lo)
        v.rY_src = array4(self.rY_src, lo)
        v.T = array4(self.T, lo)
        v.rEner = array4(self.rEner, lo)
        v.rEner_src = array4(self.rEner_src, lo)
        v.FC = array4(self.FC, lo)
        v.mask = array4(self.mask, lo) if self.mask is not None else Array4()
        return v


def _stream_ptr(stream) -> Optional[int]:
    if stream is None:
        return None
    return int(getattr(stream, "cuda_stream", stream))


def mechanism_info(name: str) -> Tuple[int, int]:
    ns, nr = C.c_int(), C.c_int()
    check(lib().pgb_mechanism_info(name.encode(), C.byref(ns), C.byref(nr)), "mechanism_info")
    return ns.value, nr.value


class ReactorGB:
    """GB300 reactor behind the ReactorBase API."""

    def __init__(self, name: str, mechanism: str, options: str = ""):
        self.name = name
        self.mechanism = mechanism
        self.options = options
        self.ns, self.nr = mechanism_info(mechanism)
        self._h = None

    def init(self, reactor_type: int = 2, ncells: int = 1) -> None:
        h = lib().pgb_reactor_create(self.name.encode(), self.mechanism.encode(), int(reactor_type),
                                     self.options.encode())
        if not h:
            raise RuntimeError(f"ReactorBase::init failed: {_lib.last_error()}")
        self._h = h

    def set_typ_vals_ode(self, typ: Sequence[float]) -> None:
        arr = (C.c_double * len(typ))(*typ)
        check(lib().pgb_reactor_set_typ_vals_ode(self._h, arr, len(typ)), "set_typ_vals_ode")

    def react(self, box: Box, rY, rY_src, T, rEner, rEner_src, FC, mask, dt_react: float,
              time: float, stream=None) -> int:
        v = BoxArrays(box, rY, rY_src, T, rEner, rEner_src, FC, mask).view()
        dt = C.c_double(dt_react)
        tm = C.c_double(time)
        return check(lib().pgb_reactor_react(self._h, C.byref(v), C.byref(dt), C.byref(tm),
                                             _stream_ptr(stream)), "react")

    def react_boxes(self, boxes: List[BoxArrays], dt_react: float, time: float = 0.0,
                    stream=None) -> None:
        arr = (BoxView * len(boxes))(*[b.view() for b in boxes])
        check(lib().pgb_reactor_react_boxes(self._h, arr, len(boxes), float(dt_react), float(time),
                                            _stream_ptr(stream)), "react_boxes")

    def stats(self) -> dict:
        s = Stats()
        check(lib().pgb_reactor_get_stats(self._h, C.byref(s)), "get_stats")
        return {"ncell": s.ncell, "nst": s.nst, "nfe": s.nfe, "nje": s.nje, "netf": s.netf,
                "ncfn": s.ncfn, "nfail": s.nfail, "max_nst": s.max_nst, "hist": list(s.hist),
                "nretry": s.nretry}

    def tuning(self) -> str:
        """The autotuner's report (gb.autotune=1), empty before the first advance."""
        buf = C.create_string_buffer(4096)
        check(min(0, lib().pgb_reactor_tuning(self._h, buf, 4096)), "tuning")
        return buf.value.decode()

    def surrogate_stats(self) -> dict:
        """Counters of the learned surrogate in the last advance (reactor made with gb.surrogate)."""
        s = _lib.SurrogateStats()
        check(lib().pgb_reactor_get_surrogate_stats(self._h, C.byref(s)), "get_surrogate_stats")
        return {n: getattr(s, n) for n, _ in _lib.SurrogateStats._fields_}

    def advance_chemistry(self, boxes: List[BoxArrays], dt: float, I_R=None, stream=None) -> None:
        """PeleLM's chemistry step on MKS arrays (rhoY kg/m^3, rhoH J/m^3, forcing kg/m^3/s and
        W/m^3): scaling, advance, back-scaling and the reaction source I_R (optional list of
        (NUM_SPECIES, nz, ny, nx) tensors, one per box) in one launch."""
        views = []
        for b, box in enumerate(boxes):
            v = _lib.ChemView()
            lo = box.box[0]
            for d in range(3):
                v.box.lo[d], v.box.hi[d] = box.box[0][d], box.box[1][d]
            v.rhoY, v.rhoY_src, v.T = array4(box.rY, lo), array4(box.rY_src, lo), array4(box.T, lo)
            v.rhoH, v.rhoH_src, v.FC = array4(box.rEner, lo), array4(box.rEner_src, lo), array4(box.FC, lo)
            v.mask = array4(box.mask, lo) if box.mask is not None else _lib.Array4()
            v.I_R = array4(I_R[b], lo) if I_R is not None else _lib.Array4()
            views.append(v)
        arr = (_lib.ChemView * len(views))(*views)
        check(lib().pgb_advance_chemistry(self._h, arr, len(views), float(dt), _stream_ptr(stream)),
              "advance_chemistry")

    def surrogate_raw(self, boxes: List[BoxArrays], out, in_rows=None) -> None:
        """Raw ensemble outputs [cell][member][n_out] (FP32 device tensor `out`) of the fused
        inference kernel, optionally its input rows [cell][k_in]; the boxes are not modified."""
        arr = (BoxView * len(boxes))(*[b.view() for b in boxes])
        check(lib().pgb_reactor_surrogate_raw(self._h, arr, len(boxes), out.data_ptr(),
                                              None if in_rows is None else in_rows.data_ptr(), None),
              "surrogate_raw")

    def close(self) -> None:
        if self._h:
            lib().pgb_reactor_close(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ReactorBase:
    """Factory with the reference's spelling: ReactorBase.create(name)."""

    @staticmethod
    def create(name: str, mechanism: str = "lidryer_syn", options: str = "") -> ReactorGB:
        if name in ("ReactorRK64", "ReactorArkode"):
            raise ValueError(f"reactor '{name}' is not provided (ReactorCvode, ReactorNull)")
        if name not in ("ReactorCvode", "ReactorNull"):
            raise ValueError(f"unknown reactor '{name}'")
        return ReactorGB(name, mechanism, options)


def typical_values_chem(rhoY_mks, T, typical_Y_val_min: float = 1e-10):
    """The typical values PeleLM hands to set_typ_vals_ode when peleLM.use_typ_vals_chem = 1.

    reset_typical_values (Source/PeleLM.cpp:1519-1545) takes, per state component, the range
    |max - min| over the field; species become mass fractions range(rhoY_k) / range(rho),
    floored at typical_Y_val_min (1e-10, :162). update_typical_values_chem (:1497-1516) then
    forms the reactor's vector in its CGS units: max(typical_Y_val_min, Y_k * rho * 1e-3) for
    the species and the temperature range for T. Inputs are cell-major: rhoY_mks (ncell, ns)
    in kg/m^3, T (ncell,) in K. Returns a list of ns + 1 floats."""
    import numpy as np
    rY = np.asarray(rhoY_mks, dtype=np.float64)
    rho = rY.sum(axis=1)

    def rng(a):
        v = abs(float(np.max(a)) - float(np.min(a)))
        return v if v > 0.0 else 0.5 * abs(float(np.max(a)) + float(np.min(a)))

    typ_rho = rng(rho)
    out = []
    for k in range(rY.shape[1]):
        typ_Y = max(rng(rY[:, k]) / typ_rho, typical_Y_val_min)
        out.append(max(typical_Y_val_min, typ_Y * typ_rho * 1.0e-3))
    out.append(rng(np.asarray(T, dtype=np.float64)))
    return out


def reaction_rates(mechanism: str, box: Box, rhoY, rhoH, T, mask, out, stream=None) -> None:
    """reactionRateRhoY over a box (MKS in/out), writing rhoYdot into `out`."""
    v = BoxArrays(box, rhoY, None, T, rhoH, None, None, mask).view()
    o = array4(out, box[0])
    check(lib().pgb_reaction_rates(mechanism.encode(), C.byref(v), C.byref(o), _stream_ptr(stream)),
          "reaction_rates")


def rhoh_to_temp(mechanism: str, box: Box, rhoY, rhoH, T, tmin=90.0, tmax=5000.0, stream=None) -> None:
    """getTfromHY over a box (MKS), T updated in place."""
    v = BoxArrays(box, rhoY, None, T, rhoH, None, None, None).view()
    check(lib().pgb_rhoh_to_temp(mechanism.encode(), C.byref(v), float(tmin), float(tmax),
                                 _stream_ptr(stream)), "rhoh_to_temp")


def heat_release(mechanism: str, box: Box, T, rhoYdot, out, stream=None) -> None:
    """HeatRelease derive over a box (MKS): out = -sum_k rhoYdot_k h_k(T) [W/m^3]."""
    from ._lib import Box as CBox
    b = CBox()
    for d in range(3):
        b.lo[d], b.hi[d] = box[0][d], box[1][d]
    check(lib().pgb_heat_release(mechanism.encode(), C.byref(b), C.byref(array4(T, box[0])),
                                 C.byref(array4(rhoYdot, box[0])), C.byref(array4(out, box[0])),
                                 _stream_ptr(stream)), "heat_release")
