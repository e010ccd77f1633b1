"""Algorithmic FP64 operation count of one reactor right-hand-side evaluation.

Counts every add, subtract, multiply and divide of the equation-level RHS
(Model.rst:227-296 kinetics/thermo plus the constant-pressure energy equation) the way the
oracle's counting scalar does (a test pins the two to be equal), with transcendentals
(exp, log, log10, pow) counted separately. One transcendental is charged
``FLOPS_PER_TRANSCENDENTAL`` flops: the flop count of the library's own FP64 exponential
(csrc/exp64.cuh: 8 FMA + 1 add + 1 multiply = 18 flops).

These counts are the "algorithmic" FP64 work the roofline divides by kernel time; the GPU
kernels execute fewer instructions for the same algorithm (folded constants, FMA).
"""
from __future__ import annotations

from typing import Tuple

from .model import Mechanism

FLOPS_PER_TRANSCENDENTAL = 18


def rhs_ops(m: Mechanism) -> Tuple[int, int]:
    ns = m.ns
    ops = 0
    trans = 1                      # lnT
    ops += ns                      # C_k = rhoY_k / W_k
    ops += 3 + 1                   # T^2, T^3, T^4, 1/T
    ops += ns * (8 + 10 + 10 + 1)  # cp/R, h/RT, s/R, g/RT per species
    # reaction loop preamble: 1/T, invT/Rc, ln(P0/RT), total concentration
    ops += 1 + 1 + 1
    trans += 1
    ops += ns
    for r in m.reactions:
        ops += 4                   # lnA + beta lnT - Ea/(Rc T)
        trans += 1                 # kf
        if r.kind != "elementary":
            ops += 2 * len(r.efficiencies)
        if r.kind == "falloff":
            ops += 4 + 2           # k0 exponent, Pr = k0 M / kinf
            trans += 1
            if r.troe:
                ops += 5
                trans += 2
                if len(r.troe) > 3:
                    ops += 2
                    trans += 1
                trans += 2         # log10 Fcent, log10 Pr
                ops += 2 + 2 + 5 + 3
                trans += 1         # pow(10, .)
            ops += 1 + 3           # 1 + Pr, kinf Pr / (1+Pr) F
        if r.reversible:
            ops += 2 * (len(r.products) + len(r.reactants))
            ops += 3
            trans += 1
        ops += sum(r.reactants.values()) + sum(r.products.values())
        ops += 4                   # q = alpha (kf Pf - kr Pp)
        ops += 2 * (len(r.reactants) + len(r.products))  # wdot accumulation
    ops += 1 + 8 * ns + 3          # RT, per-species energy terms, dT/dt
    return ops, trans


def rhs_flops(m: Mechanism) -> int:
    ops, trans = rhs_ops(m)
    return ops + FLOPS_PER_TRANSCENDENTAL * trans
