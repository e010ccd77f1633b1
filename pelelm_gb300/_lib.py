"""ctypes binding of the native library's C ABI (include/pelelm_gb300.h).

The library is the product; this module only declares its entry points. Loading fails
loudly when the library has not been built — there is no fallback implementation.
"""
from __future__ import annotations

import ctypes as C
import os

from ._build import LIB

_vp = C.c_void_p


class Array4(C.Structure):
    _fields_ = [("p", C.c_void_p), ("jstride", C.c_longlong), ("kstride", C.c_longlong),
                ("nstride", C.c_longlong), ("begin", C.c_int * 3), ("end", C.c_int * 3),
                ("ncomp", C.c_int)]


class Box(C.Structure):
    _fields_ = [("lo", C.c_int * 3), ("hi", C.c_int * 3)]


class BoxView(C.Structure):
    _fields_ = [("box", Box), ("rY", Array4), ("rY_src", Array4), ("T", Array4),
                ("rEner", Array4), ("rEner_src", Array4), ("FC", Array4), ("mask", Array4)]


class ChemView(C.Structure):
    _fields_ = [("box", Box)] + [(n, Array4) for n in ("rhoY", "rhoY_src", "T", "rhoH", "rhoH_src", "FC", "mask",
                                                        "I_R")]


class Stats(C.Structure):
    _fields_ = [("ncell", C.c_ulonglong), ("nst", C.c_ulonglong), ("nfe", C.c_ulonglong),
                ("nje", C.c_ulonglong), ("netf", C.c_ulonglong), ("ncfn", C.c_ulonglong),
                ("nfail", C.c_ulonglong), ("max_nst", C.c_ulonglong), ("hist", C.c_ulonglong * 16),
                ("nretry", C.c_ulonglong)]


class SurrogateStats(C.Structure):
    _fields_ = [(n, C.c_ulonglong) for n in ("ncell", "accept", "fallback", "ood", "mis", "cons", "ens", "neg",
                                               "audit", "audit_bad")] + \
               [("audit_max_dT", C.c_double), ("audit_max_dY", C.c_double)]


EXPORTS = {
    "pgb_version": (C.c_int, []),
    "pgb_last_error": (C.c_int, [C.c_char_p, C.c_size_t]),
    "pgb_mechanism_info": (C.c_int, [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int)]),
    "pgb_reactor_create": (_vp, [C.c_char_p, C.c_char_p, C.c_int, C.c_char_p]),
    "pgb_reactor_set_typ_vals_ode": (C.c_int, [_vp, C.POINTER(C.c_double), C.c_int]),
    "pgb_reactor_react": (C.c_int, [_vp, C.POINTER(BoxView), C.POINTER(C.c_double),
                                    C.POINTER(C.c_double), _vp]),
    "pgb_reactor_react_boxes": (C.c_int, [_vp, C.POINTER(BoxView), C.c_int, C.c_double,
                                          C.c_double, _vp]),
    "pgb_reactor_get_stats": (C.c_int, [_vp, C.POINTER(Stats)]),
    "pgb_reactor_get_surrogate_stats": (C.c_int, [_vp, C.POINTER(SurrogateStats)]),
    "pgb_surrogate_features": (C.c_int, [C.c_char_p, _vp, C.c_int, _vp, _vp]),
    "pgb_reactor_surrogate_raw": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp, _vp]),
    "pgb_heat_release": (C.c_int, [C.c_char_p, _vp, _vp, _vp, _vp, _vp]),
    "pgb_advance_chemistry": (C.c_int, [_vp, _vp, C.c_int, C.c_double, _vp]),
    "pgb_reactor_tuning": (C.c_int, [_vp, C.c_char_p, C.c_size_t]),
    "pgb_reactor_close": (None, [_vp]),
    "pgb_reaction_rates": (C.c_int, [C.c_char_p, C.POINTER(BoxView), C.POINTER(Array4), _vp]),
    "pgb_rhoh_to_temp": (C.c_int, [C.c_char_p, C.POINTER(BoxView), C.c_double, C.c_double, _vp]),
    "pgb_fp64_peak_tflops": (C.c_int, [C.c_int, C.POINTER(C.c_double)]),
    "pgb_chop_boxes": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, C.c_int]),
    "pgb_partition_boxes": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "pgb_mlp_gemm_nt": (C.c_int, [_vp, C.c_int, _vp, C.c_int, C.c_int, C.c_int, C.c_int, _vp, C.c_int,
                                  _vp, _vp, _vp, C.c_int, C.c_int, _vp]),
    "pgb_mlp_transpose_bf16": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, C.c_int, _vp]),
    "pgb_mlp_gelu_backward": (C.c_int, [_vp, _vp, _vp, _vp, C.c_longlong, _vp]),
    "pgb_mlp_mse_grad": (C.c_int, [_vp, _vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _vp]),
    "pgb_mlp_bias_grad": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp]),
    "pgb_mlp_adam": (C.c_int, [_vp, _vp, _vp, _vp, _vp, C.c_longlong, C.c_float, C.c_float, C.c_float,
                               C.c_float, C.c_int, _vp]),
    "pgb_mlp_f32_to_bf16": (C.c_int, [_vp, _vp, C.c_longlong, _vp]),
    "pgb_mlp_dup_weight_bf16": (C.c_int, [_vp, C.c_int, C.c_int, _vp, C.c_int, _vp]),
    "pgb_mlp_split_rows_bf16": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, C.c_int, C.c_int, _vp]),
    "pgb_newton_matrix": (C.c_int, [C.c_char_p, C.c_int, C.c_longlong, _vp, _vp, _vp, C.c_double, _vp,
                                    C.c_int, _vp, _vp, _vp]),
    "pgb_react_boxes_noalloc": (C.c_int, [C.c_char_p, C.POINTER(BoxView), C.c_int, C.c_double,
                                          C.c_double, C.c_double, C.c_int, C.c_int, C.c_int, _vp,
                                          C.POINTER(Stats)]),
}

_lib = None


def lib():
    """Load the native library (building it first is the caller's job: __graft_entry__.build
    or ``python -m pelelm_gb300._build``)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise RuntimeError(f"pelelm_gb300 native library missing ({LIB}); build it with "
                               "`python -m pelelm_gb300._build`")
        L = C.CDLL(LIB)
        for name, (res, args) in EXPORTS.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def last_error() -> str:
    buf = C.create_string_buffer(1024)
    lib().pgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def check(rc: int, what: str) -> int:
    if rc < 0:
        raise RuntimeError(f"{what} failed: {last_error()}")
    return rc
