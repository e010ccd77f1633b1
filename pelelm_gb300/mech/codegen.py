"""CUDA code generator for a mechanism: one header per mechanism with fully unrolled
production rates, reactor right-hand side and analytic Jacobian.

Plays the role FUEGO plays for PelePhysics (``Docs/source/manual/Model.rst:296-310``:
mechanism-specific generated rate/thermo code), written from scratch for sm_103a:

* all mechanism constants are folded into immediates (ln A, Ea/R, 1/W, NASA-7 with the
  per-species coefficient set picked by a predicated select, never a divergent branch);
* rates evaluate ln k in FP64 FMAs and take one exponential per coefficient;
* the Jacobian is a template on its arithmetic type: ``float`` recomputes every rate
  coefficient in FP32 (the inexact-Newton preconditioner), ``double`` gives the plain
  FP64 Jacobian. It writes J(i,k) through an accessor so the caller decides where the
  matrix lives (shared memory per thread).

The formulas are those of the CPU oracle (``oracle/chem_oracle.cpp``), which is the
equation-level restatement of Model.rst:227-296.
"""
from __future__ import annotations

import math
import os
from typing import Dict, List

from .model import Mechanism, R_CAL, R_ERG, P_ATM

LN10 = math.log(10.0)


def _f(x: float) -> str:
    r = repr(float(x))
    if "e" not in r and "." not in r and "inf" not in r and "nan" not in r:
        r += ".0"
    return r


class _Emitter:
    def __init__(self):
        self.lines: List[str] = []
        self.ind = 0

    def __call__(self, s: str = ""):
        self.lines.append("  " * self.ind + s if s else "")

    def text(self) -> str:
        return "\n".join(self.lines) + "\n"


def _thermo_select(e: _Emitter, m: Mechanism, prec: str):
    """Emit per-species NASA-7 coefficient selects a{k}_{i} for the current T."""
    tmids = sorted({s.Tmid for s in m.species})
    for t in tmids:
        e(f"const bool lo_{int(t)} = T < {_f(t)};")
    cast = "" if prec == "double" else "f"
    for k, s in enumerate(m.species):
        for i in range(7):
            lo, hi = s.low[i], s.high[i]
            e(f"const {prec} a{k}_{i} = lo_{int(s.Tmid)} ? {_f(lo)}{cast} : {_f(hi)}{cast};")


def _sel(lo_flag: str, lo: float, hi: float, prec: str = "double") -> str:
    """Predicated select between two folded immediates (no branch)."""
    if prec == "double":
        return f"({lo_flag} ? {_f(lo)} : {_f(hi)})"
    return f"({lo_flag} ? R({_f(lo)}) : R({_f(hi)}))"


def _g_expr(k, s, lo_flag):
    """g/RT = a0 (1-lnT) - a1 T/2 - a2 T^2/6 - a3 T^3/12 - a4 T^4/20 + a5/T - a6 (FP64, 6 FMA)."""
    L, H = s.low, s.high
    c = lambda i, f: _sel(lo_flag, L[i] * f, H[i] * f)
    return (f"fma({c(0, 1.0)}, lnT1, fma(T, fma(T, fma(T, fma(T, {c(4, -0.05)}, {c(3, -1.0 / 12.0)}), "
            f"{c(2, -1.0 / 6.0)}), {c(1, -0.5)}), fma({c(5, 1.0)}, invT, {c(6, -1.0)})))")


def _hW_expr(s, lo_flag, scale):
    """scale * h/RT (FP64, 5 FMA)."""
    L, H = s.low, s.high
    c = lambda i, f: _sel(lo_flag, L[i] * f * scale, H[i] * f * scale)
    return (f"fma(T, fma(T, fma(T, fma(T, {c(4, 0.2)}, {c(3, 0.25)}), {c(2, 1.0 / 3.0)}), {c(1, 0.5)}), "
            f"fma({c(5, 1.0)}, invT, {c(0, 1.0)}))")


def _cpW_expr(s, lo_flag, scale):
    """scale * cp/R (FP64, 4 FMA)."""
    L, H = s.low, s.high
    c = lambda i: _sel(lo_flag, L[i] * scale, H[i] * scale)
    return f"fma(T, fma(T, fma(T, fma(T, {c(4)}, {c(3)}), {c(2)}), {c(1)}), {c(0)})"


def check_supported(m: Mechanism) -> None:
    """The kernels take every reverse rate from K_c; explicit reverse Arrhenius parameters
    (CHEMKIN REV, which the reader keeps) are refused here rather than silently ignored."""
    for j, r in enumerate(m.reactions):
        if r.rev is not None:
            raise ValueError(f"{m.name}: reaction {j} ({r.equation()}) has explicit reverse parameters "
                             "(REV), which the rate kernels do not evaluate")


def gen_header(m: Mechanism) -> str:
    check_supported(m)
    ns, nr = m.ns, m.nr
    N = ns + 1
    W = [s.W for s in m.species]
    idx = {s.name: i for i, s in enumerate(m.species)}
    lnP0_R = math.log(P_ATM / R_ERG)  # ln(P0/R); ln(P0/RT) = lnP0_R - lnT
    e = _Emitter()
    guard = f"PGB_MECH_{m.name.upper()}_CUH"
    e("// GENERATED by pelelm_gb300/mech/codegen.py from pelelm_gb300/data/" + m.name + ".json.")
    e("// Do not edit. " + ("SYNTHETIC structure-matched mechanism." if m.synthetic else ""))
    e(f"#ifndef {guard}")
    e(f"#define {guard}")
    e('#include "../mech_common.cuh"')
    const_tab = constant_tables(m)
    if const_tab:
        e(f'#include "tab_{m.name}.cuh"')
    e(f'#include "tabg_{m.name}.cuh"')
    e()
    e("namespace pgb {")
    e(f"struct Mech_{m.name} {{")
    e.ind += 1
    e(f"using Tab = {'tab' if const_tab else 'tabg'}_{m.name}::Tables;  // per-thread kernels")
    e(f"using TabG = tabg_{m.name}::Tables;  // warp-per-cell kernel")
    e(f"static constexpr int NS = {ns};")
    e(f"static constexpr int NR = {nr};")
    e(f"static constexpr int N = {N};")
    e(f'static constexpr const char* NAME = "{m.name}";')
    e(f"static constexpr bool SYNTHETIC = {'true' if m.synthetic else 'false'};")
    e("// small mechanisms use the unrolled RHS / Jacobian below, larger ones the table-driven loops")
    e(f"static constexpr bool JAC_TABLE = {'true' if ns > 12 else 'false'};")
    e(f"static constexpr bool RHS_TABLE = {'true' if ns > 12 else 'false'};")
    e()
    # ---------------------------------------------------------------- molecular weights
    e("__host__ __device__ static constexpr double W(int k) {")
    e("  return " + " ".join(f"k == {k} ? {_f(w)} :" for k, w in enumerate(W)) + " 0.0;")
    e("}")
    e()
    # ---------------------------------------------------------------- thermo (mixture h, cp)
    e("// Mixture mass enthalpy [erg/g] and cp [erg/g/K] at T for mass fractions Y.")
    e("__device__ __forceinline__ static void h_cp_mix(const double T, const double* __restrict__ Y, double& h, double& cp) {")
    e.ind += 1
    e("const double invT = 1.0 / T;")
    for t in sorted({s.Tmid for s in m.species}):
        e(f"const bool lo_{int(t)} = T < {_f(t)};")
    e("double hs = 0.0, cps = 0.0;")
    for k, sp in enumerate(m.species):
        lf = f"lo_{int(sp.Tmid)}"
        e(f"hs = fma(Y[{k}], {_hW_expr(sp, lf, 1.0 / W[k])}, hs);")
        e(f"cps = fma(Y[{k}], {_cpW_expr(sp, lf, 1.0 / W[k])}, cps);")
    e(f"h = hs * ({_f(R_ERG)} * T);")
    e(f"cp = cps * {_f(R_ERG)};")
    e.ind -= 1
    e("}")
    e()
    # ---------------------------------------------------------------- FP64 rates core
    def emit_rates_fp64(with_energy: bool):
        """Emit body computing q{j} from T, lnT, invT, C{k}, g{k} (FP64)."""
        # third-body concentrations
        needM = any(r.kind != "elementary" for r in m.reactions)
        if needM:
            e("const double Ctot = " + " + ".join(f"C{k}" for k in range(ns)) + ";")
        e(f"const double lnP0RT = {_f(lnP0_R)} - lnT;")
        for j, r in enumerate(m.reactions):
            e(f"// R{j}: {r.equation()}")
            lnA = math.log(r.rate.A)
            ear = r.rate.Ea / R_CAL
            e(f"double q{j};")
            e("{")
            e.ind += 1
            e(f"const double lnkf = fma({_f(r.rate.beta)}, lnT, fma({_f(-ear)}, invT, {_f(lnA)}));")
            if r.kind != "elementary":
                terms = "Ctot"
                for sname, eff in r.efficiencies.items():
                    if eff != 1.0:
                        terms = f"fma({_f(eff - 1.0)}, C{idx[sname]}, {terms})"
                e(f"const double M = {terms};")
            if r.kind == "falloff":
                lnA0 = math.log(r.low.A)
                ear0 = r.low.Ea / R_CAL
                e(f"const double lnk0 = fma({_f(r.low.beta)}, lnT, fma({_f(-ear0)}, invT, {_f(lnA0)}));")
                # Pr = k0 M / kinf
                e("const double Pr = M * pgb_exp(lnk0 - lnkf);")
                if r.troe:
                    a, T3, T1 = r.troe[:3]
                    fc = f"fma({_f(1.0 - a)}, pgb_exp(T * {_f(-1.0 / T3)}), {_f(a)} * pgb_exp(T * {_f(-1.0 / T1)}))"
                    if len(r.troe) > 3:
                        fc = f"{fc} + pgb_exp(invT * {_f(-r.troe[3])})"
                    e(f"const double Fcent = {fc};")
                    e(f"const double lFc = pgb_log(Fcent) * {_f(1.0 / LN10)};")
                    e("const double cc = fma(-0.67, lFc, -0.4), nn = fma(-1.27, lFc, 0.75);")
                    e(f"const double lPr = pgb_log(fmax(Pr, 1e-300)) * {_f(1.0 / LN10)} + cc;")
                    e("const double f1 = lPr / fma(-0.14, lPr, nn);")
                    e(f"const double Fb = pgb_exp({_f(LN10)} * lFc / fma(f1, f1, 1.0));")
                    e("const double blend = Pr / (1.0 + Pr) * Fb;")
                else:
                    e("const double blend = Pr / (1.0 + Pr);")
                e("const double kf = pgb_exp(lnkf) * blend;")
            else:
                e("const double kf = pgb_exp(lnkf);")
            pf = " * ".join(f"C{idx[s]}" for s, nu in r.reactants.items() for _ in range(nu))
            pr = " * ".join(f"C{idx[s]}" for s, nu in r.products.items() for _ in range(nu))
            if r.reversible:
                dg = []
                for s, nu in r.products.items():
                    dg.append(("+" if nu == 1 else f"+ {nu}.0 *") + f" g{idx[s]}")
                for s, nu in r.reactants.items():
                    dg.append(("-" if nu == 1 else f"- {nu}.0 *") + f" g{idx[s]}")
                dnu = sum(r.products.values()) - sum(r.reactants.values())
                dgs = " ".join(dg).lstrip("+ ").strip()
                if dnu != 0:
                    dgs += f" - {_f(dnu)} * lnP0RT"
                # exponent capped at 700: exp stays finite, so an absent product (Pp = 0)
                # gives a zero reverse term instead of inf * 0 = NaN
                e(f"const double kr = kf * pgb_exp(fmin({dgs}, 700.0));")
                e(f"q{j} = fma(kf, {pf}, -kr * {pr});")
            else:
                e(f"q{j} = kf * {pf};")
            if r.kind == "three_body":
                e(f"q{j} *= M;")
            e.ind -= 1
            e("}")
        # production rates
        for k in range(ns):
            terms = []
            for j, r in enumerate(m.reactions):
                nu = r.products.get(m.species[k].name, 0) - r.reactants.get(m.species[k].name, 0)
                if nu != 0:
                    terms.append((nu, j))
            if not terms:
                e(f"const double wd{k} = 0.0;")
                continue
            expr = ""
            for nu, j in terms:
                if expr == "":
                    expr = (f"q{j}" if nu == 1 else (f"-q{j}" if nu == -1 else f"{_f(nu)} * q{j}"))
                else:
                    expr = (f"{expr} + q{j}" if nu == 1 else
                            (f"{expr} - q{j}" if nu == -1 else f"fma({_f(nu)}, q{j}, {expr})"))
            e(f"const double wd{k} = {expr};")

    def emit_gibbs():
        for t in sorted({s.Tmid for s in m.species}):
            e(f"const bool lo_{int(t)} = T < {_f(t)};")
        e("const double lnT1 = 1.0 - lnT;")
        for k, sp in enumerate(m.species):
            e(f"const double g{k} = {_g_expr(k, sp, f'lo_{int(sp.Tmid)}')};")

    e("// Molar production rates [mol/cm^3/s] from T and concentrations C [mol/cm^3].")
    e("__device__ __forceinline__ static void wdot(const double T, const double* __restrict__ C_, double* __restrict__ wdot_) {")
    e.ind += 1
    e("const double invT = 1.0 / T;")
    e("const double lnT = pgb_log(T);")
    for k in range(ns):
        e(f"const double C{k} = C_[{k}];")
    emit_gibbs()
    emit_rates_fp64(False)
    for k in range(ns):
        e(f"wdot_[{k}] = wd{k};")
    e.ind -= 1
    e("}")
    e()
    e("// Reactor RHS (constant-pressure RhoH): y = [rhoY_k (g/cm^3), T], F = rhoY forcing,")
    e("// Fh = rho h forcing. ydot_k = W_k wdot_k + F_k; dT/dt = (Fh - sum h_k ydot_k) / (rho cp).")
    e("__device__ __forceinline__ static void rhs(const double* __restrict__ y, const double* __restrict__ F, const double Fh, double* __restrict__ ydot) {")
    e.ind += 1
    e(f"const double T = y[{ns}];")
    e("const double invT = 1.0 / T;")
    e("const double lnT = pgb_log(T);")
    for k in range(ns):
        e(f"const double C{k} = y[{k}] * {_f(1.0 / W[k])};")
    emit_gibbs()
    emit_rates_fp64(True)
    e("double hs = 0.0, rcp = 0.0;")
    for k, sp in enumerate(m.species):
        lf = f"lo_{int(sp.Tmid)}"
        e(f"{{ const double wm = fma(wd{k}, {_f(W[k])}, F[{k}]); ydot[{k}] = wm;")
        e(f"  hs = fma({_hW_expr(sp, lf, 1.0 / W[k])}, wm, hs);")
        e(f"  rcp = fma(y[{k}], {_cpW_expr(sp, lf, R_ERG / W[k])}, rcp); }}")
    e(f"ydot[{ns}] = fma(-hs, {_f(R_ERG)} * T, Fh) / rcp;")
    e.ind -= 1
    e("}")
    e()
    # ---------------------------------------------------------------- Jacobian template
    e("// Analytic Jacobian d ydot / d y in arithmetic type R, written through J(i, k).")
    e("// Falloff blending factors are held frozen in the [M] and T derivatives.")
    e("template <class R, class Acc>")
    e("__device__ __forceinline__ static void jac(const double* __restrict__ y, const double* __restrict__ Fd, const double Fhd, Acc J) {")
    e.ind += 1
    e(f"const R T = (R)y[{ns}];")
    e("const R invT = R(1) / T;")
    e("const R lnT = pgb_logT<R>(T);")
    e("const R T2 = T * T, T3 = T2 * T;")
    for k in range(ns):
        e(f"const R C{k} = (R)(y[{k}] * {_f(1.0 / W[k])});")
    # thermo in R
    tmids = sorted({s.Tmid for s in m.species})
    for t in tmids:
        e(f"const bool lo_{int(t)} = T < R({_f(t)});")
    for k, s in enumerate(m.species):
        for i in range(7):
            e(f"const R a{k}_{i} = lo_{int(s.Tmid)} ? R({_f(s.low[i])}) : R({_f(s.high[i])});")
    e("const R lnT1 = R(1) - lnT;")
    for k in range(ns):
        e(f"const R g{k} = a{k}_0 * lnT1 + T * (a{k}_1 * R(-0.5) + T * (a{k}_2 * R(-1.0 / 6.0) + T * (a{k}_3 * R(-1.0 / 12.0) + T * a{k}_4 * R(-0.05)))) + a{k}_5 * invT - a{k}_6;")
        e(f"const R h{k} = a{k}_0 + T * (a{k}_1 * R(0.5) + T * (a{k}_2 * R(1.0 / 3.0) + T * (a{k}_3 * R(0.25) + T * a{k}_4 * R(0.2)))) + a{k}_5 * invT;")
        e(f"const R cp{k} = a{k}_0 + T * (a{k}_1 + T * (a{k}_2 + T * (a{k}_3 + T * a{k}_4)));")
        e(f"const R dcp{k} = a{k}_1 + T * (R(2) * a{k}_2 + T * (R(3) * a{k}_3 + T * R(4) * a{k}_4));")
    e("for (int i = 0; i < N; ++i)")
    e("  for (int k = 0; k < N; ++k) J(i, k) = R(0);")
    needM = any(r.kind != "elementary" for r in m.reactions)
    if needM:
        e("const R Ctot = " + " + ".join(f"C{k}" for k in range(ns)) + ";")
    e(f"const R lnP0RT = R({_f(lnP0_R)}) - lnT;")
    for k in range(ns):
        e(f"R wd{k} = R(0);")
    for k in range(ns):
        e(f"R dT{k} = R(0);")
    for j, r in enumerate(m.reactions):
        e(f"// R{j}: {r.equation()}")
        e("{")
        e.ind += 1
        lnA = math.log(r.rate.A)
        ear = r.rate.Ea / R_CAL
        e(f"const R lnkf_inf = R({_f(r.rate.beta)}) * lnT + R({_f(-ear)}) * invT + R({_f(lnA)});")
        e(f"R dlnkf = (R({_f(r.rate.beta)}) + R({_f(ear)}) * invT) * invT;")
        if r.kind != "elementary":
            terms = "Ctot"
            for sname, eff in r.efficiencies.items():
                if eff != 1.0:
                    terms = f"{terms} + R({_f(eff - 1.0)}) * C{idx[sname]}"
            e(f"const R M = {terms};")
        if r.kind == "falloff":
            lnA0 = math.log(r.low.A)
            ear0 = r.low.Ea / R_CAL
            e(f"const R lnk0 = R({_f(r.low.beta)}) * lnT + R({_f(-ear0)}) * invT + R({_f(lnA0)});")
            e(f"const R dlnk0 = (R({_f(r.low.beta)}) + R({_f(ear0)}) * invT) * invT;")
            e("const R k0 = pgb_expT<R>(lnk0);")
            e("const R kinf = pgb_expT<R>(lnkf_inf);")
            e("const R Pr = M * pgb_expT<R>(lnk0 - lnkf_inf);")
            if r.troe:
                a, T3, T1 = r.troe[:3]
                fc = f"R({_f(1.0 - a)}) * pgb_expT<R>(T * R({_f(-1.0 / T3)})) + R({_f(a)}) * pgb_expT<R>(T * R({_f(-1.0 / T1)}))"
                if len(r.troe) > 3:
                    fc += f" + pgb_expT<R>(invT * R({_f(-r.troe[3])}))"
                e(f"const R Fcent = {fc};")
                e(f"const R lFc = pgb_logT<R>(Fcent) * R({_f(1.0 / LN10)});")
                e("const R cc = R(-0.4) - R(0.67) * lFc, nn = R(0.75) - R(1.27) * lFc;")
                e(f"const R lPr = pgb_logT<R>(Pr > R(1e-30) ? Pr : R(1e-30)) * R({_f(1.0 / LN10)}) + cc;")
                e("const R f1 = lPr / (nn - R(0.14) * lPr);")
                e(f"const R Fb = pgb_expT<R>(R({_f(LN10)}) * lFc / (R(1) + f1 * f1));")
            else:
                e("const R Fb = R(1);")
            e("const R onePr = R(1) + Pr;")
            e("const R kf = kinf * Pr / onePr * Fb;")
            e("const R dkeff_dM = Fb * k0 / (onePr * onePr);")
            e("dlnkf = dlnkf + (dlnk0 - dlnkf) / onePr;")
        else:
            e("const R kf = pgb_expT<R>(lnkf_inf);")
        pf_f = [idx[s] for s, nu in r.reactants.items() for _ in range(nu)]
        pr_f = [idx[s] for s, nu in r.products.items() for _ in range(nu)]
        e("const R Pf = " + " * ".join(f"C{k}" for k in pf_f) + ";")
        e("const R Pp = " + " * ".join(f"C{k}" for k in pr_f) + ";")
        dnu = sum(r.products.values()) - sum(r.reactants.values())
        if r.reversible:
            dg, dh = [], []
            for s, nu in r.products.items():
                dg.append(f"+ R({nu}) * g{idx[s]}")
                dh.append(f"+ R({nu}) * h{idx[s]}")
            for s, nu in r.reactants.items():
                dg.append(f"- R({nu}) * g{idx[s]}")
                dh.append(f"- R({nu}) * h{idx[s]}")
            dgs = " ".join(dg)
            if dnu != 0:
                dgs += f" - R({dnu}) * lnP0RT"
            e(f"const R kr = kf * pgb_expT<R>(fmin(R(0) {dgs}, R(700)));")
            e(f"const R dlnkr = dlnkf - (R(0) {' '.join(dh)} - R({dnu})) * invT;")
        else:
            e("const R kr = R(0);")
            e("const R dlnkr = R(0);")
        alpha = "M" if r.kind == "three_body" else "R(1)"
        e(f"const R alpha = {alpha};")
        e("const R q = alpha * (kf * Pf - kr * Pp);")
        e("const R dqdT = alpha * (kf * dlnkf * Pf - kr * dlnkr * Pp);")
        # partials dq/dC_k
        dq: Dict[int, List[str]] = {}

        def partials(side_list, coef):
            uniq = sorted(set(side_list))
            for k in uniq:
                nu = side_list.count(k)
                others = list(side_list)
                others.remove(k)
                term = f"{coef}" + (f" * R({nu})" if nu > 1 else "") + "".join(f" * C{o}" for o in others)
                dq.setdefault(k, []).append(term)

        partials(pf_f, "alpha * kf")
        if r.reversible:
            partials(pr_f, "-alpha * kr")
        if r.kind == "three_body":
            e("const R base = kf * Pf - kr * Pp;")
        elif r.kind == "falloff":
            e("const R base = dkeff_dM * (Pf - (kf > R(0) ? kr / kf : R(0)) * Pp);")
        for k, terms in dq.items():
            e(f"const R dq{k} = " + " + ".join(terms) + ";")
        nus = {}
        for s, nu in r.reactants.items():
            nus[idx[s]] = nus.get(idx[s], 0) - nu
        for s, nu in r.products.items():
            nus[idx[s]] = nus.get(idx[s], 0) + nu
        for i, nu in nus.items():
            if nu == 0:
                continue
            e(f"wd{i} += R({nu}) * q;")
            e(f"dT{i} += R({nu}) * dqdT;")
            for k in dq:
                e(f"J({i}, {k}) += R({_f(nu * W[i] / W[k])}) * dq{k};")
            if r.kind != "elementary":
                effs = {idx[s]: eff for s, eff in r.efficiencies.items()}
                for k in range(ns):
                    eff = effs.get(k, 1.0)
                    if eff != 0.0:
                        e(f"J({i}, {k}) += R({_f(nu * W[i] / W[k] * eff)}) * base;")
        e.ind -= 1
        e("}")
    # temperature column and energy row
    e("R Dm = R(0), dDm = R(0), Q = (R)Fhd;")
    for k in range(ns):
        e(f"const R wm{k} = wd{k} * R({_f(W[k])}) + (R)Fd[{k}];")
        e(f"const R hm{k} = h{k} * R({_f(R_ERG / W[k])}) * T;")
        e(f"const R cpm{k} = cp{k} * R({_f(R_ERG / W[k])});")
        e(f"Dm += (R)y[{k}] * cpm{k};")
        e(f"dDm += (R)y[{k}] * dcp{k} * R({_f(R_ERG / W[k])});")
        e(f"Q -= hm{k} * wm{k};")
        e(f"J({k}, {ns}) = R({_f(W[k])}) * dT{k};")
    e("const R invD = R(1) / Dm;")
    e("const R QD2 = Q * invD * invD;")
    for k in range(ns):
        terms = " + ".join(f"hm{i} * J({i}, {k})" for i in range(ns))
        e(f"J({ns}, {k}) = -({terms}) * invD - QD2 * cpm{k};")
    terms = " + ".join(f"cpm{i} * wm{i} + hm{i} * J({i}, {ns})" for i in range(ns))
    e(f"J({ns}, {ns}) = -({terms}) * invD - QD2 * dDm;")
    e.ind -= 1
    e("}")
    e.ind -= 1
    e("};")
    e("}  // namespace pgb")
    e(f"#endif  // {guard}")
    return e.text()


def main(outdir: str, names=("lidryer_syn", "drm19_syn", "gri_syn")):
    from ..workloads import load_mechanism
    os.makedirs(outdir, exist_ok=True)
    for n in names:
        m = load_mechanism(n)
        text = gen_header(m)
        path = os.path.join(outdir, f"mech_{n}.cuh")
        if os.path.exists(path):
            with open(path) as f:
                if f.read() == text:
                    continue  # unchanged: keep the timestamp so the library is not rebuilt
        with open(path, "w") as f:
            f.write(text)


if __name__ == "__main__":
    import sys
    here = os.path.dirname(os.path.abspath(__file__))
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(here, "..", "csrc", "gen"))


# ---------------------------------------------------------------------------- tables
def rx_packed(rx, ns: int) -> list:
    """The four words of each reaction's TabRxPk record (mech_tables.cuh): x = kind | rev << 2 |
    nr << 3 | np << 5 | (dnu + 8) << 7 | (tb + 1) << 11 | (troe + 1) << 22; y, z = the reactant and
    product species slots, 10 bits each; w = 0."""
    assert ns <= 1024, "species index fields of the packed reaction record are 10 bits"
    out = []
    for (_, _, _, kind, rev, rs, ps, dnu, tb, tr) in rx:
        assert -8 <= dnu <= 7 and tb + 1 < 2048 and tr + 1 < 1024
        x = kind | rev << 2 | len(rs) << 3 | len(ps) << 5 | (dnu + 8) << 7 | (tb + 1) << 11 | (tr + 1) << 22
        y = sum(k << (10 * s_) for s_, k in enumerate(rs))
        z = sum(k << (10 * s_) for s_, k in enumerate(ps))
        out.append((x, y, z, 0))
    return out


def gen_tables(m: Mechanism, space: str = "constant") -> str:
    """Mechanism tables for the table-driven kernels: per-species W, NASA-7 sets, per-reaction
    Arrhenius data, stoichiometry as species slots (a species with coefficient 2 occupies two
    slots), sparse third-body efficiencies and Troe parameters.

    space "constant": __constant__ arrays in namespace tab_<name> (per-thread kernels: every lane
    reads the same entry, a constant-cache broadcast). space "global": read-only global arrays in
    namespace tabg_<name> (warp-per-cell kernels: lanes read different entries through L1; also
    the only choice when the tables exceed the 64 KB constant bank), plus the species-major list
    of the reactions each species takes part in with its net coefficient (production rates as a
    gather)."""
    check_supported(m)
    glob = space == "global"
    qual = "__device__ const" if glob else "__device__ __constant__"
    nsname = f"tabg_{m.name}" if glob else f"tab_{m.name}"
    ns = m.ns
    idx = {s.name: i for i, s in enumerate(m.species)}
    tb_rows, troe_rows = [], []
    rx = []
    for r in m.reactions:
        rs = [idx[s] for s, nu in r.reactants.items() for _ in range(nu)]
        ps = [idx[s] for s, nu in r.products.items() for _ in range(nu)]
        assert len(rs) <= 3 and len(ps) <= 3
        kind = {"elementary": 0, "three_body": 1, "falloff": 2}[r.kind]
        tb = -1
        if r.kind != "elementary":
            tb = len(tb_rows)
            effs = [(idx[s], e - 1.0) for s, e in r.efficiencies.items() if e != 1.0]
            tb_rows.append(effs)
        tr = -1
        if r.kind == "falloff":
            tr = len(troe_rows)
            lnA0 = math.log(r.low.A)
            t = r.troe or []
            troe_rows.append((lnA0, r.low.beta, -r.low.Ea / R_CAL, len(t),
                              (1.0 - t[0]) if t else 0.0, (-1.0 / t[1]) if t else 0.0,
                              t[0] if t else 0.0, (-1.0 / t[2]) if t else 0.0,
                              (-t[3]) if len(t) > 3 else 0.0))
        dnu = sum(r.products.values()) - sum(r.reactants.values())
        rx.append((math.log(r.rate.A), r.rate.beta, -r.rate.Ea / R_CAL, kind, int(r.reversible),
                   rs, ps, dnu, tb, tr))
    if glob:
        # warp-per-cell kernels give consecutive reactions to the lanes of a warp: group them by
        # kind (elementary, third-body, falloff) so a 32-reaction pass rarely mixes code paths
        order = sorted(range(len(rx)), key=lambda j: (rx[j][3], j))
        rx = [rx[j] for j in order]
    maxeff = max([len(t) for t in tb_rows] + [1])
    e = _Emitter()
    e(f"// GENERATED by pelelm_gb300/mech/codegen.py (tables, {space} memory) from pelelm_gb300/data/{m.name}.json.")
    guard = f"PGB_{nsname.upper()}_CUH"
    e(f"#ifndef {guard}")
    e(f"#define {guard}")
    e('#include "../mech_tables.cuh"')
    e("namespace pgb {")
    e(f"namespace {nsname} {{")
    e(f"constexpr int NS = {ns}, NR = {m.nr}, NTB = {max(1, len(tb_rows))}, NTROE = {max(1, len(troe_rows))}, MAXEFF = {maxeff};")
    for R, suf, cast in (("double", "D", lambda x: _f(x)), ("float", "F", lambda x: _f(x) + "f")):
        e(f"{qual} TabSpecies<{R}> kSpecies{suf}[NS] = {{")
        def gco(a):
            return [a[0], -a[1] / 2, -a[2] / 6, -a[3] / 12, -a[4] / 20, a[5], -a[6]]

        def hco(a):
            return [a[0], a[1] / 2, a[2] / 3, a[3] / 4, a[4] / 5, a[5]]

        for sp_ in m.species:
            arrs = [sp_.low, sp_.high, gco(sp_.low), gco(sp_.high), hco(sp_.low), hco(sp_.high)]
            body = ", ".join("{" + ", ".join(cast(a_) for a_ in arr) + "}" for arr in arrs)
            e(f"  {{{cast(sp_.W)}, {cast(1.0 / sp_.W)}, {cast(sp_.Tmid)}, {body}}},")
        e("};")
        e(f"{qual} TabReaction<{R}> kReactions{suf}[NR] = {{")
        for (lnA, beta, mear, kind, rev, rs, ps, dnu, tb, tr) in rx:
            rsl = ", ".join(str(x) for x in (rs + [0, 0, 0])[:3])
            psl = ", ".join(str(x) for x in (ps + [0, 0, 0])[:3])
            e(f"  {{{cast(lnA)}, {cast(beta)}, {cast(mear)}, {kind}, {rev}, {len(rs)}, {len(ps)}, {{{rsl}}}, {{{psl}}}, {dnu}, {tb}, {tr}}},")
        e("};")
        e(f"{qual} TabThirdBody<{R}> kThirdBody{suf}[NTB] = {{")
        if not tb_rows:
            e(f"  {{0, {{0}}, {{{cast(0.0)}}}}},")
        for effs in tb_rows:
            sp = ", ".join(str(k) for k, _ in effs) or "0"
            ev = ", ".join(cast(v) for _, v in effs) or cast(0.0)
            e(f"  {{{len(effs)}, {{{sp}}}, {{{ev}}}}},")
        e("};")
        e(f"{qual} TabTroe<{R}> kTroe{suf}[NTROE] = {{")
        if not troe_rows:
            e("  {" + ", ".join([cast(0.0)] * 3 + ["0"] + [cast(0.0)] * 5) + "},")
        for t in troe_rows:
            e("  {" + ", ".join(cast(v) if isinstance(v, float) else str(v) for v in t) + "},")
        e("};")
    if glob:
        # species-major reaction lists: species k takes part in reactions kSpRxJ[kSpRxOff[k]..
        # kSpRxOff[k+1]) with net molar coefficient kSpRxNu (products minus reactants), in
        # reaction order
        off, jj, nu = [0], [], []
        for k in range(ns):
            for j, (_, _, _, _, _, rs_, ps_, _, _, _) in enumerate(rx):
                net = ps_.count(k) - rs_.count(k)
                if net != 0:
                    jj.append(j)
                    nu.append(float(net))
            off.append(len(jj))
        # Jacobian contribution program of the cooperative setup (warp and lane-group kernels):
        # every nonzero species entry A[i][k] (and T-column entry A[i][NS]) of the analytic
        # Jacobian with its ordered terms. A term of reaction j adds c * v to its entry, c =
        # -+W_i / W_k (-+W_i in the T column; minus for a reactant row slot) and v the sum of the
        # stored partials of j that its code selects. Terms keep the order of the reaction walk
        # they replace: reactions ascending, then the row slots of the reaction. Entries go to
        # the 32 lanes largest first, to the lane with the fewest terms so far; each lane's terms
        # are stored interleaved (term t of lane l at 32 t + l, lanes padded with empty terms to
        # the longest) so a warp reads one contiguous line per load. Only the 4-byte codes are
        # streamed per setup: W_i / W_k comes from the species table at an entry's first term,
        # and a collider efficiency is read only where it differs from 1.
        # code bits: 0-8 reaction (table order), 9-20 entry i * (N + 1) + k, 21 dq/dT (T column),
        # 22-24 / 25-27 the reactant / product slots of j holding species k, 28 the collider
        # term dq/d[M] times the efficiency of k, 29 last term of its entry (store the sum), 30
        # first term of its entry, 31 efficiency different from 1 (read it); the sign of c is
        # carried by bit 29 of a separate bit plane (kJacNeg, one bit per term).
        N = ns + 1
        LDA = N + 1
        assert m.nr <= 512 and N * LDA <= 4096, "program code fields too narrow for this mechanism"
        prog = {}
        for j, (_, _, _, kind_, _, rs_, ps_, _, tb_, _) in enumerate(rx):
            effs = dict(tb_rows[tb_]) if kind_ != 0 else {}
            rows = [(i, True) for i in rs_] + [(i, False) for i in ps_]
            cols = sorted(set(rs_) | set(ps_)) if kind_ == 0 else list(range(ns))
            for k in cols:
                code = j
                for s_, sk in enumerate(rs_):
                    if sk == k:
                        code |= 1 << (22 + s_)
                for s_, sk in enumerate(ps_):
                    if sk == k:
                        code |= 1 << (25 + s_)
                em1 = None
                if kind_ != 0:
                    code |= 1 << 28
                    em1 = effs.get(k)
                    if em1 is not None:
                        code |= 1 << 31
                for (i, isr) in rows:
                    prog.setdefault((i, k), []).append((code, isr, em1))
            for (i, isr) in rows:
                prog.setdefault((i, ns), []).append((j | (1 << 21), isr, None))
        ents = sorted(prog.items(), key=lambda kv: (-len(kv[1]), kv[0]))
        lanes = [[] for _ in range(32)]
        load = [0] * 32
        for key, terms in ents:
            l_ = min(range(32), key=lambda x: (load[x], x))
            lanes[l_].append((key, terms))
            load[l_] += len(terms)
        T = max(load)
        codes = [0] * (32 * T)
        neg = [0] * T  # bit l of word t: term t of lane l has a reactant row slot (c < 0)
        effD = ["1.0"] * (32 * T)
        effF = ["1.0f"] * (32 * T)
        for l_ in range(32):
            t = 0
            for (i, k), terms in lanes[l_]:
                for n_, (code, isr, em1) in enumerate(terms):
                    pos = 32 * t + l_
                    flags = ((1 << 29) if n_ == len(terms) - 1 else 0) | ((1 << 30) if n_ == 0 else 0)
                    codes[pos] = (code | ((i * LDA + k) << 9) | flags) & 0xFFFFFFFF
                    if isr:
                        neg[t] |= 1 << l_
                    if em1 is not None:
                        effD[pos] = f"(1.0 + {_f(em1)})"
                        effF[pos] = f"(1.0f + {_f(em1)}f)"
                    t += 1
        e(f"constexpr int NJT = {T};  // program terms per lane (padded)")
        e(f"{qual} unsigned kJacC[32 * NJT] = {{{', '.join(str(x) + 'u' for x in codes)}}};")
        e(f"{qual} unsigned kJacNeg[NJT] = {{{', '.join(str(x) + 'u' for x in neg)}}};")
        e(f"{qual} double kJacEffD[32 * NJT] = {{{', '.join(effD)}}};")
        e(f"{qual} float kJacEffF[32 * NJT] = {{{', '.join(effF)}}};")
        # packed reaction records of the FP64 rate of progress (TabRxArr / TabRxPk)
        e(f"{qual} TabRxArr kRxArr[NR] = {{")
        for (lnA, beta, mear, *_r) in rx:
            e(f"  {{{_f(lnA)}, {_f(beta)}, {_f(mear)}, 0.0}},")
        e("};")
        e(f"{qual} TabRxPk kRxPk[NR] = {{")
        for w in rx_packed(rx, ns):
            e("  {" + ", ".join(f"{v}u" for v in w) + "},")
        e("};")
        e(f"constexpr int NSPRX = {len(jj)};")
        e(f"{qual} int kSpRxOff[NS + 1] = {{{', '.join(str(x) for x in off)}}};")
        e(f"{qual} int kSpRxJ[NSPRX] = {{{', '.join(str(x) for x in jj)}}};")
        e(f"{qual} double kSpRxNu[NSPRX] = {{{', '.join(_f(x) for x in nu)}}};")
    e("struct Tables {")
    e(f"  static constexpr int NS = {ns}, NR = {m.nr};")
    if glob:
        e("  __device__ static int sprx_begin(int k) { return kSpRxOff[k]; }")
        e("  __device__ static int sprx_end(int k) { return kSpRxOff[k + 1]; }")
        e("  __device__ static int sprx_j(int e) { return kSpRxJ[e]; }")
        e("  __device__ static double sprx_nu(int e) { return kSpRxNu[e]; }")
        e("  __device__ static const TabRxArr& rx_arr(int j) { return kRxArr[j]; }")
        e("  __device__ static TabRxPk rx_pk(int j) { return kRxPk[j]; }")
        e("  static constexpr int JAC_TERMS = NJT;")
        e("  __device__ static unsigned jac_code(int c) { return kJacC[c]; }")
        e("  __device__ static unsigned jac_neg(int t) { return kJacNeg[t]; }")
        e("  template <class R> __device__ static R jac_eff(int c) {")
        e("    if constexpr (sizeof(R) == sizeof(double)) return kJacEffD[c]; else return kJacEffF[c];")
        e("  }")
    for nm, typ, arr in (("sp", "TabSpecies", "kSpecies"), ("rx", "TabReaction", "kReactions"),
                         ("tb", "TabThirdBody", "kThirdBody"), ("troe", "TabTroe", "kTroe")):
        e(f"  template <class R> __device__ static const {typ}<R>& {nm}(int i) {{")
        e(f"    if constexpr (sizeof(R) == sizeof(double)) return {arr}D[i]; else return {arr}F[i];")
        e("  }")
    e("};")
    e(f"}}  // namespace {nsname}")
    e("}  // namespace pgb")
    e(f"#endif  // {guard}")
    return e.text()


def kernel_family(m: Mechanism) -> str:
    """Which persistent BDF kernels a mechanism gets: "thread" (cell per thread and per warp)
    up to 12 species, "group" (cell per thread, per lane group and per warp) while the ODE size
    stays within one warp's lanes (N <= 32), else "warp" only (one cell's state no longer fits a
    thread)."""
    if m.ns <= 12:
        return "thread"
    return "group" if m.ns + 1 <= 32 else "warp"


def constant_tables(m: Mechanism) -> bool:
    """Tables in the 64 KB constant bank for the per-thread kernels (mechanisms that have them);
    every mechanism also gets the global-memory tables of the lane-group and warp kernels."""
    return kernel_family(m) != "warp"


def write_tables(outdir: str, names=("lidryer_syn", "drm19_syn", "gri_syn")):
    from ..workloads import load_mechanism
    for n in names:
        m = load_mechanism(n)
        outs = [(f"tabg_{n}.cuh", gen_tables(m, "global"))]
        if constant_tables(m):
            outs.append((f"tab_{n}.cuh", gen_tables(m, "constant")))
        for fname, text in outs:
            path = os.path.join(outdir, fname)
            if os.path.exists(path):
                with open(path) as f:
                    if f.read() == text:
                        continue
            with open(path, "w") as f:
                f.write(text)


# ---------------------------------------------------------------------------- registry
_ENTRY_MACRO = {"thread": "PGB_MECH_ENTRY", "group": "PGB_MECH_ENTRY_GROUP", "warp": "PGB_MECH_ENTRY_WARP"}


def write_units(outdir: str, names) -> list:
    """One translation unit per mechanism (its kernels and registry entry) and the registry list
    included by csrc/reactor.cu; returns the unit paths. Files are rewritten only on change."""
    from ..workloads import load_mechanism

    def put(path, text):
        if os.path.exists(path):
            with open(path) as f:
                if f.read() == text:
                    return
        with open(path, "w") as f:
            f.write(text)

    units = []
    reg = ["// GENERATED by pelelm_gb300/mech/codegen.py from the mechanisms in pelelm_gb300/data/.",
           "// Registry of the compiled mechanisms (one unit_<name>.cu each), included by reactor.cu.",
           "namespace pgb_host {"]
    for n in names:
        m = load_mechanism(n)
        fam = kernel_family(m)
        text = "\n".join([
            f"// GENERATED by pelelm_gb300/mech/codegen.py from pelelm_gb300/data/{n}.json.",
            f"// Kernels of mechanism {n} ({m.ns} species, {m.nr} reactions; BDF kernel family: {fam}) and",
            "// its registry entry.",
            f'#include "mech_{n}.cuh"',
            '#include "../reactor_registry.cuh"',
            "",
            "namespace pgb_host {",
            f"extern const MechEntry kEntry_{n} = {_ENTRY_MACRO[fam]}(pgb::Mech_{n});",
            "}  // namespace pgb_host",
            ""])
        path = os.path.join(outdir, f"unit_{n}.cu")
        put(path, text)
        units.append(path)
        reg.append(f"extern const MechEntry kEntry_{n};")
    reg.append("}  // namespace pgb_host")
    reg.append("#define PGB_MECH_LIST " + ", ".join(f"&::pgb_host::kEntry_{n}" for n in names))
    put(os.path.join(outdir, "mech_registry.inc"), "\n".join(reg) + "\n")
    return units
