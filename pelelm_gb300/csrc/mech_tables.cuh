// Constant-memory mechanism tables and the table-driven analytic Jacobian.
//
// The Jacobian of the reactor RHS (d ydot / d y for y = [rhoY_k, T]) as a compact loop over
// reactions: every lane of a warp reads the same table entry (constant-cache broadcast), so
// the loop costs one small code block instead of a fully unrolled expansion per reaction —
// the per-pass instruction footprint of the persistent BDF kernel stays inside the SM's
// instruction cache. The equations are those of the oracle's analytic Jacobian
// (oracle/chem_oracle.cpp, reactor_jac): mass-action partials, third-body and falloff
// [M]-derivatives with the Troe blending factor held frozen, temperature derivatives through
// d ln k / dT and van 't Hoff for K_c, and the constant-pressure energy row.
#ifndef PGB_MECH_TABLES_CUH
#define PGB_MECH_TABLES_CUH

#include "mech_common.cuh"

namespace pgb {

// Table entry types, one instantiation per arithmetic type so the FP32 Jacobian never
// converts double constants (a double->float convert occupies the FP64 pipe on GB300).
template <class R>
struct TabSpecies {
  R W, invW, Tmid;
  R lo[7], hi[7];    // NASA-7 a1..a7 below / above Tmid
  R glo[7], ghi[7];  // g/RT = c0 (1 - lnT) + T(c1 + T(c2 + T(c3 + T c4))) + c5/T + c6
  R hlo[6], hhi[6];  // h/RT = c0 + T(c1 + T(c2 + T(c3 + T c4))) + c5/T
};

template <class R>
struct TabReaction {
  R lnA, beta, mEaR;      // ln A, beta, -Ea/R (k or k_inf)
  int kind, rev, nr, np;  // kind 0 elementary, 1 third-body, 2 falloff
  int rs[3], ps[3];       // species slots (a coefficient 2 occupies two slots)
  int dnu, tb, troe;      // sum(nu'') - sum(nu'), third-body row or -1, falloff row or -1
};

// The FP64 rate of progress of the warp and lane-group kernels reads a reaction through two
// aligned records instead of the fields of TabReaction one by one (the same values): the
// Arrhenius triple, and the integer fields packed in four words —
//   x: kind (bits 0-1), rev (2), nr (3-4), np (5-6), dnu + 8 (7-10), tb + 1 (11-21),
//      troe + 1 (22-31);  y: rs[0..2], z: ps[0..2], 10 bits each;  w: 0.
struct __align__(32) TabRxArr {
  double lnA, beta, mEaR, pad;
};
struct __align__(16) TabRxPk {
  unsigned x, y, z, w;
};

template <class R>
struct TabThirdBody {
  int n;
  int sp[8];
  R effm1[8];  // efficiency - 1 of the listed species (others have efficiency 1)
};

template <class R>
struct TabTroe {
  R lnA0, beta0, mEa0R;  // k_0
  int ntroe;             // 0 Lindemann, 3 or 4 Troe parameters
  R one_m_a, m_invT3, a, m_invT1, m_T2;
};

constexpr double kLnP0OverR = -4.407418589020958;  // ln(1 atm / R) in CGS (ln(P0/RT) = this - ln T)
constexpr double kRerg = 8.31446261815324e7;        // erg/mol/K

namespace jac_detail {
template <class R>
__device__ __forceinline__ void nasa(const TabSpecies<R>& s, R T, R invT, R lnT1, R& gRT, R& hRT,
                                     R& cpR, R& dcpR) {
  const bool lo = T < s.Tmid;
  R a[7];
#pragma unroll
  for (int i = 0; i < 7; ++i) a[i] = lo ? s.lo[i] : s.hi[i];
  cpR = a[0] + T * (a[1] + T * (a[2] + T * (a[3] + T * a[4])));
  dcpR = a[1] + T * (R(2) * a[2] + T * (R(3) * a[3] + T * R(4) * a[4]));
  hRT = a[0] + T * (a[1] * R(0.5) + T * (a[2] * R(1.0 / 3.0) + T * (a[3] * R(0.25) + T * a[4] * R(0.2)))) +
        a[5] * invT;
  gRT = a[0] * lnT1 + T * (a[1] * R(-0.5) + T * (a[2] * R(-1.0 / 6.0) + T * (a[3] * R(-1.0 / 12.0) + T * a[4] * R(-0.05)))) +
        a[5] * invT - a[6];
}
}  // namespace jac_detail

// J(i,k) = d ydot_i / d y_k in type R. y: state (FP64, registers); Fr(k): rhoY forcing; Fh: rho h
// forcing; Cs(k): per-thread scratch of NS values (holds the concentrations).
template <class Tab, class R, class Acc, class Scr, class Frc>
__device__ void jac_table(const double* y, Frc Fr, double Fh, Acc J, Scr Cs) {
  using namespace jac_detail;
  constexpr int NS = Tab::NS;
  const R T = (R)y[NS];
  const R invT = R(1) / T;
  const R lnT = pgb_logT<R>(T);
  const R lnT1 = R(1) - lnT;
  const R lnP0RT = R(kLnP0OverR) - lnT;
  const R RT = R(kRerg) * T;
  R Ctot = R(0);
  for (int k = 0; k < NS; ++k) {
    const R c = (R)y[k] * Tab::template sp<R>(k).invW;
    Cs(k) = c;
    Ctot += c;
  }
  for (int i = 0; i <= NS; ++i)
    for (int k = 0; k <= NS; ++k) J(i, k) = R(0);
  R Qw = R(0), cpw = R(0);  // sum_i h_i W_i wdot_i and sum_i cp_i W_i wdot_i (mass units)

#pragma unroll 1
  for (int j = 0; j < Tab::NR; ++j) {
    const TabReaction<R>& r = Tab::template rx<R>(j);
    const R lnkinf = r.beta * lnT + r.mEaR * invT + r.lnA;
    R dlnkf = (r.beta - r.mEaR * invT) * invT;
    R kf = pgb_expT<R>(lnkinf);
    R M = R(1), alpha = R(1), dkeff_dM = R(0);
    if (r.tb >= 0) {
      const TabThirdBody<R>& t = Tab::template tb<R>(r.tb);
      M = Ctot;
      for (int e = 0; e < t.n; ++e) M += t.effm1[e] * Cs(t.sp[e]);
      if (r.kind == 1) alpha = M;
    }
    if (r.kind == 2) {
      const TabTroe<R>& f = Tab::template troe<R>(r.troe);
      const R lnk0 = f.beta0 * lnT + f.mEa0R * invT + f.lnA0;
      const R dlnk0 = (f.beta0 - f.mEa0R * invT) * invT;
      const R k0 = pgb_expT<R>(lnk0);
      const R Pr = M * pgb_expT<R>(lnk0 - lnkinf);
      R Fb = R(1);
      if (f.ntroe > 0) {
        R Fcent = f.one_m_a * pgb_expT<R>(T * f.m_invT3) + f.a * pgb_expT<R>(T * f.m_invT1);
        if (f.ntroe > 3) Fcent += pgb_expT<R>(f.m_T2 * invT);
        const R lFc = pgb_logT<R>(Fcent) * R(0.4342944819032518);
        const R cc = R(-0.4) - R(0.67) * lFc, nn = R(0.75) - R(1.27) * lFc;
        const R lPr = pgb_logT<R>(Pr > R(1e-30) ? Pr : R(1e-30)) * R(0.4342944819032518) + cc;
        const R f1 = lPr / (nn - R(0.14) * lPr);
        Fb = pgb_expT<R>(R(2.302585092994046) * lFc / (R(1) + f1 * f1));
      }
      const R onePr = R(1) + Pr;
      kf = kf * Pr / onePr * Fb;
      dkeff_dM = Fb * k0 / (onePr * onePr);
      dlnkf = dlnkf + (dlnk0 - dlnkf) / onePr;
    }
    // concentration products and the partial of each slot product
    R cr[3], cp[3];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      cr[s] = s < r.nr ? Cs(r.rs[s]) : R(1);
      cp[s] = s < r.np ? Cs(r.ps[s]) : R(1);
    }
    const R Pf = cr[0] * cr[1] * cr[2];
    const R Pp = cp[0] * cp[1] * cp[2];
    R kr = R(0), dlnkr = R(0);
    if (r.rev) {
      R dG = -(R)r.dnu * lnP0RT, dH = R(0);
      for (int s = 0; s < r.np; ++s) {
        R g, h, c, d;
        nasa<R>(Tab::template sp<R>(r.ps[s]), T, invT, lnT1, g, h, c, d);
        dG += g;
        dH += h;
      }
      for (int s = 0; s < r.nr; ++s) {
        R g, h, c, d;
        nasa<R>(Tab::template sp<R>(r.rs[s]), T, invT, lnT1, g, h, c, d);
        dG -= g;
        dH -= h;
      }
      kr = kf * pgb_expT<R>(fmin(dG, R(700)));  // finite: Pp = 0 gives 0, not NaN
      dlnkr = dlnkf - (dH - (R)r.dnu) * invT;
    }
    const R q = alpha * (kf * Pf - kr * Pp);
    const R dqdT = alpha * (kf * dlnkf * Pf - kr * dlnkr * Pp);
    R pr_part[3], pp_part[3];
#pragma unroll
    for (int s = 0; s < 3; ++s) {
      pr_part[s] = alpha * kf * (s == 0 ? cr[1] * cr[2] : s == 1 ? cr[0] * cr[2] : cr[0] * cr[1]);
      pp_part[s] = -alpha * kr * (s == 0 ? cp[1] * cp[2] : s == 1 ? cp[0] * cp[2] : cp[0] * cp[1]);
    }
    R base = R(0);
    if (r.kind == 1) base = kf * Pf - kr * Pp;
    else if (r.kind == 2) base = dkeff_dM * (Pf - (kf > R(0) ? kr / kf : R(0)) * Pp);
    // rows: every reactant slot loses one, every product slot gains one
#pragma unroll 1
    for (int row = 0; row < r.nr + r.np; ++row) {
      const bool isr = row < r.nr;
      const int i = isr ? r.rs[row] : r.ps[row - r.nr];
      const R sgnW = (isr ? R(-1) : R(1)) * Tab::template sp<R>(i).W;
      J(i, NS) += sgnW * dqdT;
      {
        R g, h, c, d;
        nasa<R>(Tab::template sp<R>(i), T, invT, lnT1, g, h, c, d);
        // mass-based h_i W_i = hRT RT and cp_i W_i = cpR R
        Qw += (isr ? -q : q) * h * RT;
        cpw += (isr ? -q : q) * c * R(kRerg);
      }
      for (int s = 0; s < r.nr; ++s) {
        const int k = r.rs[s];
        J(i, k) += sgnW * Tab::template sp<R>(k).invW * pr_part[s];
      }
      for (int s = 0; s < r.np; ++s) {
        const int k = r.ps[s];
        J(i, k) += sgnW * Tab::template sp<R>(k).invW * pp_part[s];
      }
      if (r.kind != 0) {
        const R sb = sgnW * base;
        for (int k = 0; k < NS; ++k) J(i, k) += sb * Tab::template sp<R>(k).invW;
        const TabThirdBody<R>& t = Tab::template tb<R>(r.tb);
        for (int e = 0; e < t.n; ++e) J(i, t.sp[e]) += sb * Tab::template sp<R>(t.sp[e]).invW * t.effm1[e];
      }
    }
  }
  // constant-pressure energy row: dT/dt = (Fh - sum h_k wm_k) / (rho cp)
  R D = R(0), dD = R(0), Q = (R)Fh - Qw, cpwm = cpw;
  for (int k = 0; k < NS; ++k) {
    R g, h, c, d;
    nasa<R>(Tab::template sp<R>(k), T, invT, lnT1, g, h, c, d);
    const R iw = Tab::template sp<R>(k).invW;
    const R cpm = c * R(kRerg) * iw, hm = h * RT * iw;
    const R yk = (R)y[k];
    const R fk = (R)Fr(k);
    D += yk * cpm;
    dD += yk * d * R(kRerg) * iw;
    Q -= hm * fk;
    cpwm += cpm * fk;
  }
  // row NS accumulates sum_i h_i J(i, k) for every column k (including the T column)
  for (int i = 0; i < NS; ++i) {
    R g, h, c, d;
    nasa<R>(Tab::template sp<R>(i), T, invT, lnT1, g, h, c, d);
    const R hm = h * RT * Tab::template sp<R>(i).invW;
    for (int k = 0; k <= NS; ++k) J(NS, k) += hm * J(i, k);
  }
  const R invD = R(1) / D;
  const R QD2 = Q * invD * invD;
  for (int k = 0; k < NS; ++k) {
    R g, h, c, d;
    nasa<R>(Tab::template sp<R>(k), T, invT, lnT1, g, h, c, d);
    const R cpm = c * R(kRerg) * Tab::template sp<R>(k).invW;
    J(NS, k) = -J(NS, k) * invD - QD2 * cpm;
  }
  J(NS, NS) = -(J(NS, NS) + cpwm) * invD - QD2 * dD;
}

// Reactor RHS in FP64 as a loop over reactions (the same equations as the generated unrolled
// RHS and the oracle's reactor_rhs): for mechanisms too large to unroll. Per-species loops are
// unrolled (NS is a compile-time constant); concentrations, Gibbs energies and the molar
// production accumulators live in the per-thread scratch accessors Cs, Gs, Ws (dynamic
// indices inside the reaction loop).
template <class Tab, class Frc, class SC, class SG, class SW>
__device__ __forceinline__ void rhs_table(const double* y, Frc Fr, double Fh, double* ydot, SC Cs,
                                          SG Gs, SW Ws) {
  constexpr int NS = Tab::NS;
  const double T = y[NS];
  const double invT = 1.0 / T;
  const double lnT = pgb_log64(T);
  const double lnT1 = 1.0 - lnT;
  const double lnP0RT = kLnP0OverR - lnT;
  double Ctot = 0.0;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const TabSpecies<double>& s = Tab::template sp<double>(k);
    const double c = y[k] * s.invW;
    Cs(k) = c;
    Ctot += c;
    const double* g = T < s.Tmid ? s.glo : s.ghi;
    Gs(k) = fma(g[0], lnT1, fma(T, fma(T, fma(T, fma(T, g[4], g[3]), g[2]), g[1]), fma(g[5], invT, g[6])));
    Ws(k) = 0.0;
  }
#pragma unroll 1
  for (int j = 0; j < Tab::NR; ++j) {
    const TabReaction<double>& r = Tab::template rx<double>(j);
    const double lnkf = fma(r.beta, lnT, fma(r.mEaR, invT, r.lnA));
    double kf = pgb_exp64(lnkf);
    double M = 1.0;
    if (r.tb >= 0) {
      const TabThirdBody<double>& t = Tab::template tb<double>(r.tb);
      M = Ctot;
      for (int e = 0; e < t.n; ++e) M = fma(t.effm1[e], Cs(t.sp[e]), M);
    }
    if (r.kind == 2) {
      const TabTroe<double>& f = Tab::template troe<double>(r.troe);
      const double lnk0 = fma(f.beta0, lnT, fma(f.mEa0R, invT, f.lnA0));
      const double Pr = M * pgb_exp64(lnk0 - lnkf);
      double blend = Pr / (1.0 + Pr);
      if (f.ntroe > 0) {
        double Fcent = fma(f.one_m_a, pgb_exp64(T * f.m_invT3), f.a * pgb_exp64(T * f.m_invT1));
        if (f.ntroe > 3) Fcent += pgb_exp64(invT * f.m_T2);
        const double lFc = pgb_log64(Fcent) * 0.4342944819032518;
        const double cc = fma(-0.67, lFc, -0.4), nn = fma(-1.27, lFc, 0.75);
        const double lPr = pgb_log64(fmax(Pr, 1e-300)) * 0.4342944819032518 + cc;
        const double f1 = lPr / fma(-0.14, lPr, nn);
        blend *= pgb_exp64(2.302585092994046 * lFc / fma(f1, f1, 1.0));
      }
      kf *= blend;
    }
    double Pf = 1.0, Pp = 1.0;
    for (int s = 0; s < r.nr; ++s) Pf *= Cs(r.rs[s]);
    for (int s = 0; s < r.np; ++s) Pp *= Cs(r.ps[s]);
    double q;
    if (r.rev) {
      double dG = -r.dnu * lnP0RT;
      for (int s = 0; s < r.np; ++s) dG += Gs(r.ps[s]);
      for (int s = 0; s < r.nr; ++s) dG -= Gs(r.rs[s]);
      const double kr = kf * pgb_exp64(fmin(dG, 700.0));  // finite: Pp = 0 gives 0, not NaN
      q = fma(kf, Pf, -kr * Pp);
    } else {
      q = kf * Pf;
    }
    if (r.kind == 1) q *= M;
    for (int s = 0; s < r.nr; ++s) Ws(r.rs[s]) -= q;
    for (int s = 0; s < r.np; ++s) Ws(r.ps[s]) += q;
  }
  // dT/dt = (Fh - sum h_k ydot_k) / (rho cp)
  double hs = 0.0, rcp = 0.0;
#pragma unroll
  for (int k = 0; k < NS; ++k) {
    const TabSpecies<double>& s = Tab::template sp<double>(k);
    const double wm = fma(Ws(k), s.W, (double)Fr(k));
    ydot[k] = wm;
    const bool lo = T < s.Tmid;
    const double* a = lo ? s.lo : s.hi;
    const double* hc = lo ? s.hlo : s.hhi;
    const double hRT = fma(T, fma(T, fma(T, fma(T, hc[4], hc[3]), hc[2]), hc[1]), fma(hc[5], invT, hc[0]));
    const double cpR = fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
    hs = fma(hRT * s.invW, wm, hs);
    rcp = fma(y[k] * s.invW, cpR, rcp);
  }
  ydot[NS] = fma(-hs, kRerg * T, Fh) / (rcp * kRerg);
}

}  // namespace pgb

#endif  // PGB_MECH_TABLES_CUH
