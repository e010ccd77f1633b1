// Persistent, work-stealing, warp-per-cell BDF reactor kernel for mechanisms whose per-cell state
// no longer fits a thread: the default for drm19-sized mechanisms (21 species, 84 reactions) and
// the only mapping for GRI-Mech-sized ones (53 species, 325 reactions, N = 54 unknowns).
//
// Same contract and algorithm as bdf_kernel.cuh (the PelePhysics reactor called at
// Source/PeleLM.cpp:5752; CVODE-class fixed-leading-coefficient variable-order Nordsieck BDF,
// modified Newton with analytic Jacobian and dense partial-pivot LU, CVODE's documented
// step/order heuristics): each warp runs the step loop of oracle/bdf_oracle.cpp for one cell at a
// time, with the length-N vectors split over the lanes (element i in lane i % 32, slot i / 32).
//
// GB300 mapping:
//  * the scalar step logic runs redundantly in every lane (uniform values, no divergence): an
//    FP64 warp instruction costs the same whatever its active mask, so this is free next to a
//    lane-parallel right-hand side;
//  * RHS: lanes over species (concentrations, g/RT, h, cp), then over reactions (rates of
//    progress, from global-memory tables read through L1: lanes read different entries), then
//    over species again gathering their reactions (species-major lists: a deterministic order,
//    no atomics), with warp-shuffle sums for the energy closure;
//  * Jacobian (type JR: FP32 in mixed precision): NASA-7 terms once per species, per-reaction
//    partials lane-parallel, then an assembly in reaction order with lanes over columns (each
//    lane owns its columns, so the result does not depend on scheduling); constant-pressure
//    energy row by column;
//  * LU and triangular solves: lanes own rows; pivot search by warp arg-max (FP32: one max-
//    reduction over the |a| bit patterns); matrix rows padded to N+1 so a column access is
//    bank-conflict free;
//  * per-warp state (Nordsieck history, forcing, rates, matrix) in shared memory; a warp takes
//    the next cell index with one atomic when its cell is done (work stealing across all boxes);
//  * with a retry list (mixed precision), a failed cell is listed and left untouched for the
//    FP64 pass that follows on the same stream.
#ifndef PGB_BDF_WARP_KERNEL_CUH
#define PGB_BDF_WARP_KERNEL_CUH

#include "bdf_kernel.cuh"
#include "mech_tables.cuh"

namespace pgb {

namespace wbdf {
constexpr int RXW = 8;  // Jacobian scratch per reaction: dq/dT, 3 reactant partials, 3 product partials, [M] partial
}

// Shared memory of one warp (one cell) for mechanism M and Jacobian type JR: the FP64 state
// (Nordsieck history, forcing, l, tau), one scratch region and the matrix. The scratch region
// holds the RHS scratch (concentrations, g/RT, rates of progress) inside warp_rhs and the setup
// scratch (per-reaction partials, NASA-7 terms) inside warp_setup: never both live.
template <class M>
__host__ __device__ constexpr int bdf_warp_state_bytes() {
  return (((QMAX + 2) * M::N + M::N + (QMAX + 1) + (QMAX + 2)) * 8 + 15) / 16 * 16;
}
template <class M, class JR>
__host__ __device__ constexpr int bdf_warp_scratch_bytes() {
  constexpr int NS = M::NS, NR = M::NR;
  constexpr int rhs = (2 * NS + NR) * 8, setup = (wbdf::RXW * NR + 4 * NS) * (int)sizeof(JR);
  return ((rhs > setup ? rhs : setup) + 15) / 16 * 16;
}
template <class M, class JR>
__host__ __device__ constexpr int bdf_warp_smem_per_warp() {
  constexpr int N = M::N;
  constexpr int nj = N * (N + 1) + N;
  return (bdf_warp_state_bytes<M>() + bdf_warp_scratch_bytes<M, JR>() + nj * (int)sizeof(JR) + N * 4 + 15) / 16 * 16;
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ float warp_sum(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}
__device__ __forceinline__ double warp_max(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}

// The lane-distributed part of a length-N vector (element i in lane i % 32, slot i / 32).
template <class M>
struct WVec {
  double v[(M::N + 31) / 32];
};

// Rate of progress of reaction j (table order) at one state, FP64: the equations of the table
// RHS in mech_tables.cuh (Arrhenius forward rate, third-body and Lindemann/Troe fall-off
// factors, reverse rate from K_c with the exponent capped at 700), the same operations in the
// same order. Shared by the warp and lane-group right-hand sides; the reaction's data comes
// from its two packed records (TabRxArr, TabRxPk: three loads instead of one per field).
template <class Tab>
__device__ __forceinline__ double rate_of_progress(int j, double T, double invT, double lnT, double lnP0RT,
                                                   double Ctot, const double* CS, const double* GS) {
  const TabRxArr& ar = Tab::rx_arr(j);
  const TabRxPk pk = Tab::rx_pk(j);
  const int kind = pk.x & 3u, nr = (pk.x >> 3) & 3u, np = (pk.x >> 5) & 3u;
  const bool rev = (pk.x >> 2) & 1u;
  const int dnu = (int)((pk.x >> 7) & 15u) - 8, tbi = (int)((pk.x >> 11) & 2047u) - 1;
  const int troe = (int)(pk.x >> 22) - 1;
  auto rs = [&](int s) { return (int)((pk.y >> (10 * s)) & 1023u); };
  auto ps = [&](int s) { return (int)((pk.z >> (10 * s)) & 1023u); };
  const double lnkf = fma(ar.beta, lnT, fma(ar.mEaR, invT, ar.lnA));
  double kf = pgb_exp64(lnkf);
  double Mc = 1.0;
  if (tbi >= 0) {
    const TabThirdBody<double>& tb = Tab::template tb<double>(tbi);
    Mc = Ctot;
#pragma unroll
    for (int e = 0; e < 8; ++e)
      if (e < tb.n) Mc = fma(tb.effm1[e], CS[tb.sp[e]], Mc);
  }
  if (kind == 2) {
    const TabTroe<double>& fo = Tab::template troe<double>(troe);
    const double lnk0 = fma(fo.beta0, lnT, fma(fo.mEa0R, invT, fo.lnA0));
    const double Pr = Mc * pgb_exp64(lnk0 - lnkf);
    double blend = Pr / (1.0 + Pr);
    if (fo.ntroe > 0) {
      double Fcent = fma(fo.one_m_a, pgb_exp64(T * fo.m_invT3), fo.a * pgb_exp64(T * fo.m_invT1));
      if (fo.ntroe > 3) Fcent += pgb_exp64(invT * fo.m_T2);
      const double lFc = pgb_log64(Fcent) * 0.4342944819032518;
      const double cc = fma(-0.67, lFc, -0.4), nn = fma(-1.27, lFc, 0.75);
      const double lPr = pgb_log64(fmax(Pr, 1e-300)) * 0.4342944819032518 + cc;
      const double f1 = lPr / fma(-0.14, lPr, nn);
      blend *= pgb_exp64(2.302585092994046 * lFc / fma(f1, f1, 1.0));
    }
    kf *= blend;
  }
  double Pf = 1.0, Pp = 1.0;
#pragma unroll
  for (int s = 0; s < 3; ++s) if (s < nr) Pf *= CS[rs(s)];
#pragma unroll
  for (int s = 0; s < 3; ++s) if (s < np) Pp *= CS[ps(s)];
  double q;
  if (rev) {
    double dG = -dnu * lnP0RT;
#pragma unroll
    for (int s = 0; s < 3; ++s) if (s < np) dG += GS[ps(s)];
#pragma unroll
    for (int s = 0; s < 3; ++s) if (s < nr) dG -= GS[rs(s)];
    const double kr = kf * pgb_exp64(fmin(dG, 700.0));  // finite: Pp = 0 gives 0, not NaN
    q = fma(kf, Pf, -kr * Pp);
  } else {
    q = kf * Pf;
  }
  if (kind == 1) q *= Mc;
  return q;
}

// Right-hand side f = [W_k wdot_k + F_k, dT/dt] at y, one warp cooperating (see the kernel
// below). One non-inlined copy serves every call site: the step loop calls it from five places
// and inlined copies of this exp/log-heavy body overflow the instruction cache.
template <class M>
__device__ __noinline__ WVec<M> warp_rhs(const WVec<M> yv, double* CS, double* GS, double* QS,
                                         const double* FRC) {
  using Tab = typename M::TabG;
  constexpr int N = M::N, NS = M::NS, NR = M::NR;
  constexpr int R = (N + 31) / 32;
  const int lane = threadIdx.x & 31;
  auto idx = [&](int r) { return lane + 32 * r; };
  const double (&y)[R] = yv.v;
  WVec<M> fv;
  double (&f)[R] = fv.v;
  auto bcast = [&](const double (&v)[R], int i) -> double {
    return __shfl_sync(0xffffffffu, v[i >> 5], i & 31);
  };
  const double T = bcast(y, NS);
  const double invT = 1.0 / T;
  const double lnT = pgb_log64(T);
  const double lnT1 = 1.0 - lnT;
  const double lnP0RT = kLnP0OverR - lnT;
  double c_loc = 0.0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int k = idx(r);
    if (k < NS) {
      const TabSpecies<double>& s = Tab::template sp<double>(k);
      const double c = y[r] * s.invW;
      CS[k] = c;
      c_loc += c;
      const double* g = T < s.Tmid ? s.glo : s.ghi;
      GS[k] = fma(g[0], lnT1, fma(T, fma(T, fma(T, fma(T, g[4], g[3]), g[2]), g[1]), fma(g[5], invT, g[6])));
    }
  }
  const double Ctot = warp_sum(c_loc);
  __syncwarp();
  for (int j = lane; j < NR; j += 32) {
    QS[j] = rate_of_progress<Tab>(j, T, invT, lnT, lnP0RT, Ctot, CS, GS);
  }
  __syncwarp();
  double hs = 0.0, rcp = 0.0;
#pragma unroll
  for (int r = 0; r < R; ++r) {
    const int k = idx(r);
    f[r] = 0.0;
    if (k < NS) {
      double wdot = 0.0;
      const int e1 = Tab::sprx_end(k);
#pragma unroll 4
      for (int e = Tab::sprx_begin(k); e < e1; ++e) wdot = fma(Tab::sprx_nu(e), QS[Tab::sprx_j(e)], wdot);
      const TabSpecies<double>& s = Tab::template sp<double>(k);
      const double wm = fma(wdot, s.W, FRC[k]);
      f[r] = wm;
      const bool lo = T < s.Tmid;
      const double* a = lo ? s.lo : s.hi;
      const double* hc = lo ? s.hlo : s.hhi;
      const double hRT = fma(T, fma(T, fma(T, fma(T, hc[4], hc[3]), hc[2]), hc[1]), fma(hc[5], invT, hc[0]));
      const double cpR = fma(T, fma(T, fma(T, fma(T, a[4], a[3]), a[2]), a[1]), a[0]);
      hs = fma(hRT * s.invW, wm, hs);
      rcp = fma(y[r] * s.invW, cpR, rcp);
    }
  }
  hs = warp_sum(hs);
  rcp = warp_sum(rcp);
  const double fT = fma(-hs, kRerg * T, FRC[NS]) / (rcp * kRerg);
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (idx(r) == NS) f[r] = fT;
  __syncwarp();  // CS/GS/QS are reused by the next evaluation
  return fv;
}

// Jacobian (equations of jac_table, mech_tables.cuh) and partial-pivot LU of I - gamma J in
// shared memory, one warp cooperating. False: singular. With FACTOR false it stops after the
// Jacobian, which A then holds (the diagnostic entry point). Inlined: each kernel calls it from
// one place, so inlining adds no copy and removes the call's register save and restore
// (measured: lane-group kernel +5 %, warp kernel +1 %).
template <class M, class JR, bool FACTOR = true>
__device__ __forceinline__ bool warp_setup(const WVec<M> yv, const double gamma, const double* FRC, JR* A,
                                        JR* XS, JR* RX, JR* TH, int* PIV) {
  using Tab = typename M::TabG;
  constexpr int N = M::N, NS = M::NS, NR = M::NR;
  constexpr int R = (N + 31) / 32;
  constexpr int LDA = N + 1;
  const int lane = threadIdx.x & 31;
  auto idx = [&](int r) { return lane + 32 * r; };
  auto bcast = [&](const double (&v)[R], int i) -> double {
    return __shfl_sync(0xffffffffu, v[i >> 5], i & 31);
  };
  auto jacobian = [&](const double (&y)[R]) {
    using namespace jac_detail;
    const JR T = (JR)bcast(y, NS);
    const JR invT = JR(1) / T;
    const JR lnT = pgb_logT<JR>(T);
    const JR lnT1 = JR(1) - lnT;
    const JR lnP0RT = JR(kLnP0OverR) - lnT;
    const JR RT = JR(kRerg) * T;
    // per species, once: concentration (the solve vector is free during the setup) and the
    // NASA-7 terms g/RT, h/RT, cp/R, d(cp/R)/dT that the reaction and energy terms reuse
    JR* TG = TH;
    JR* TH_ = TH + NS;
    JR* TC = TH + 2 * NS;
    JR* TD = TH + 3 * NS;
    JR c_loc = JR(0);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int k = idx(r);
      if (k < NS) {
        const JR c = (JR)y[r] * Tab::template sp<JR>(k).invW;
        XS[k] = c;
        c_loc += c;
        JR g, h, cp, d;
        nasa<JR>(Tab::template sp<JR>(k), T, invT, lnT1, g, h, cp, d);
        TG[k] = g;
        TH_[k] = h;
        TC[k] = cp;
        TD[k] = d;
      }
    }
    const JR Ctot = warp_sum(c_loc);
    for (int e = lane; e < N * LDA; e += 32) A[e] = JR(0);
    __syncwarp();
    // (1) per-reaction partials, lanes over reactions; energy-closure sums
    JR Qw = JR(0), cpw = JR(0);
    for (int j = lane; j < NR; j += 32) {
      const TabReaction<JR>& r = Tab::template rx<JR>(j);
      const JR lnkinf = r.beta * lnT + r.mEaR * invT + r.lnA;
      JR dlnkf = (r.beta - r.mEaR * invT) * invT;
      JR kf = pgb_expT<JR>(lnkinf);
      JR Mc = JR(1), alpha = JR(1), dkeff_dM = JR(0);
      if (r.tb >= 0) {
        const TabThirdBody<JR>& t = Tab::template tb<JR>(r.tb);
        Mc = Ctot;
#pragma unroll
        for (int e = 0; e < 8; ++e)
          if (e < t.n) Mc += t.effm1[e] * XS[t.sp[e]];
        if (r.kind == 1) alpha = Mc;
      }
      if (r.kind == 2) {
        const TabTroe<JR>& fo = Tab::template troe<JR>(r.troe);
        const JR lnk0 = fo.beta0 * lnT + fo.mEa0R * invT + fo.lnA0;
        const JR dlnk0 = (fo.beta0 - fo.mEa0R * invT) * invT;
        const JR k0 = pgb_expT<JR>(lnk0);
        const JR Pr = Mc * pgb_expT<JR>(lnk0 - lnkinf);
        JR Fb = JR(1);
        if (fo.ntroe > 0) {
          JR Fcent = fo.one_m_a * pgb_expT<JR>(T * fo.m_invT3) + fo.a * pgb_expT<JR>(T * fo.m_invT1);
          if (fo.ntroe > 3) Fcent += pgb_expT<JR>(fo.m_T2 * invT);
          const JR lFc = pgb_logT<JR>(Fcent) * JR(0.4342944819032518);
          const JR cc = JR(-0.4) - JR(0.67) * lFc, nn = JR(0.75) - JR(1.27) * lFc;
          const JR lPr = pgb_logT<JR>(Pr > JR(1e-30) ? Pr : JR(1e-30)) * JR(0.4342944819032518) + cc;
          const JR f1 = lPr / (nn - JR(0.14) * lPr);
          Fb = pgb_expT<JR>(JR(2.302585092994046) * lFc / (JR(1) + f1 * f1));
        }
        const JR onePr = JR(1) + Pr;
        kf = kf * Pr / onePr * Fb;
        dkeff_dM = Fb * k0 / (onePr * onePr);
        dlnkf = dlnkf + (dlnk0 - dlnkf) / onePr;
      }
      JR cr[3], cp[3];
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        cr[s] = s < r.nr ? XS[r.rs[s]] : JR(1);
        cp[s] = s < r.np ? XS[r.ps[s]] : JR(1);
      }
      const JR Pf = cr[0] * cr[1] * cr[2];
      const JR Pp = cp[0] * cp[1] * cp[2];
      JR kr = JR(0), dlnkr = JR(0);
      if (r.rev) {
        JR dG = -(JR)r.dnu * lnP0RT, dH = JR(0);
#pragma unroll
        for (int s = 0; s < 3; ++s)
          if (s < r.np) {
            dG += TG[r.ps[s]];
            dH += TH_[r.ps[s]];
          }
#pragma unroll
        for (int s = 0; s < 3; ++s)
          if (s < r.nr) {
            dG -= TG[r.rs[s]];
            dH -= TH_[r.rs[s]];
          }
        kr = kf * pgb_expT<JR>(fmin(dG, JR(700)));
        dlnkr = dlnkf - (dH - (JR)r.dnu) * invT;
      }
      const JR q = alpha * (kf * Pf - kr * Pp);
      JR* out = RX + j * wbdf::RXW;
      out[0] = alpha * (kf * dlnkf * Pf - kr * dlnkr * Pp);
#pragma unroll
      for (int s = 0; s < 3; ++s) {
        out[1 + s] = alpha * kf * (s == 0 ? cr[1] * cr[2] : s == 1 ? cr[0] * cr[2] : cr[0] * cr[1]);
        out[4 + s] = -alpha * kr * (s == 0 ? cp[1] * cp[2] : s == 1 ? cp[0] * cp[2] : cp[0] * cp[1]);
      }
      JR bm = JR(0);
      if (r.kind == 1) bm = kf * Pf - kr * Pp;
      else if (r.kind == 2) bm = dkeff_dM * (Pf - (kf > JR(0) ? kr / kf : JR(0)) * Pp);
      out[7] = bm;
#pragma unroll
      for (int row = 0; row < 6; ++row)
        if (row < r.nr + r.np) {
          const bool isr = row < r.nr;
          const int i = isr ? r.rs[row] : r.ps[row - r.nr];
          Qw += (isr ? -q : q) * TH_[i] * RT;
          cpw += (isr ? -q : q) * TC[i] * JR(kRerg);
        }
    }
    Qw = warp_sum(Qw);
    cpw = warp_sum(cpw);
    __syncwarp();
    // (2) assembly by the generated contribution program: each lane owns whole entries A[i][k]
    // (species rows; k = NS: the T column) and sums their terms in a register, in the order of
    // the reaction walk (reactions ascending, then row slots): a term of reaction j is c v,
    // c = -+W_i / W_k (-+W_i in the T column) and v the partials of j that land in column k
    // (dq/dT in the T column). The lanes' 4-byte term codes are interleaved in the table (one
    // contiguous line per warp load); each entry has one writer, so the result does not depend
    // on the lane schedule.
    {
      JR acc = JR(0), w = JR(0);
#pragma unroll 1
      for (int t = 0; t < Tab::JAC_TERMS; ++t) {
        const int c = 32 * t + lane;
        const unsigned code = Tab::jac_code(c);
        const bool neg = (Tab::jac_neg(t) >> lane) & 1u;
        if (code & (1u << 30)) {  // first term of an entry: its coefficient magnitude
          const int tg = (code >> 9) & 0xfff;
          const int i = tg / LDA, k = tg - i * LDA;
          const JR wi = Tab::template sp<JR>(i).W;
          w = (k == NS) ? wi : wi * Tab::template sp<JR>(k).invW;
        }
        const JR* pj = RX + (code & 0x1ff) * wbdf::RXW;
        const bool tcol = (code & (1u << 21)) != 0;
        JR v;
        if (tcol) {
          v = pj[0];
        } else {
          v = JR(0);
#pragma unroll
          for (int q = 0; q < 3; ++q)
            if (code & (1u << (22 + q))) v += pj[1 + q];
#pragma unroll
          for (int q = 0; q < 3; ++q)
            if (code & (1u << (25 + q))) v += pj[4 + q];
          if (code & (1u << 28)) v += pj[7] * ((code & (1u << 31)) ? Tab::template jac_eff<JR>(c) : JR(1));
        }
        if (tcol || v != JR(0)) acc += (neg ? -w : w) * v;
        if (code & (1u << 29)) {  // last term of the entry
          A[(code >> 9) & 0xfff] = acc;
          acc = JR(0);
        }
      }
    }
    __syncwarp();
    // (3) constant-pressure energy row: dT/dt = (Fh - sum h_k wm_k) / (rho cp)
    JR D = JR(0), dD = JR(0), Qf = JR(0), cpf = JR(0);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int k = idx(r);
      if (k < NS) {
        const JR h = TH_[k], c = TC[k], d = TD[k];
        const JR iw = Tab::template sp<JR>(k).invW;
        const JR cpm = c * JR(kRerg) * iw, hm = h * RT * iw;
        const JR yk = (JR)y[r];
        const JR fk = (JR)FRC[k];
        D += yk * cpm;
        dD += yk * d * JR(kRerg) * iw;
        Qf -= hm * fk;
        cpf += cpm * fk;
      }
    }
    D = warp_sum(D);
    dD = warp_sum(dD);
    const JR Q = (JR)FRC[NS] - Qw + warp_sum(Qf);
    const JR cpwm = cpw + warp_sum(cpf);
    const JR invD = JR(1) / D;
    const JR QD2 = Q * invD * invD;
#pragma unroll
    for (int cc = 0; cc < R; ++cc) {
      const int k = idx(cc);
      if (k > NS) continue;
      JR acc = JR(0);
#pragma unroll 1
      for (int i = 0; i < NS; ++i) acc += TH_[i] * RT * Tab::template sp<JR>(i).invW * A[i * LDA + k];
      if (k < NS) {
        A[NS * LDA + k] = -acc * invD - QD2 * TC[k] * JR(kRerg) * Tab::template sp<JR>(k).invW;
      } else {
        A[NS * LDA + NS] = -(acc + cpwm) * invD - QD2 * dD;
      }
    }
    __syncwarp();
  };

  // ---- M = I - gamma J, partial-pivot LU in place (trailing swaps), reciprocal pivots ----
  auto factor = [&](double gamma) -> bool {
    const JR g = (JR)gamma;
    for (int e = lane; e < N * LDA; e += 32) {
      const int i = e / LDA, k = e - i * LDA;
      if (k < N) A[e] = (i == k ? JR(1) : JR(0)) - g * A[e];
    }
    __syncwarp();
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
      // pivot: first row of largest |a_ik|, i >= k (NaN never wins; none above 0: singular)
      int p = N;
      if constexpr (sizeof(JR) == sizeof(float)) {
        // a non-negative float orders as its bit pattern: one warp max-reduction, then the
        // lowest row holding the maximum from the lane ballots (rows lane + 32 r, r ascending)
        unsigned bits[R], m = 0u;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int i = idx(r);
          unsigned b = 0u;
          if (i >= k && i < N) {
            const float v = fabsf(A[i * LDA + k]);
            if (v == v) b = __float_as_uint(v);
          }
          bits[r] = b;
          m = max(m, b);
        }
        m = __reduce_max_sync(0xffffffffu, m);
        if (m == 0u) return false;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const unsigned bal = __ballot_sync(0xffffffffu, bits[r] == m);
          if (p == N && bal) p = 32 * r + __ffs(bal) - 1;
        }
      } else {
        JR best = JR(-1);
        int bi = N;
#pragma unroll
        for (int r = 0; r < R; ++r) {
          const int i = idx(r);
          if (i >= k && i < N) {
            const JR v = fabs(A[i * LDA + k]);
            if (v > best) { best = v; bi = i; }
          }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          const JR ob = __shfl_xor_sync(0xffffffffu, best, o);
          const int oi = __shfl_xor_sync(0xffffffffu, bi, o);
          if (ob > best || (ob == best && oi < bi)) { best = ob; bi = oi; }
        }
        if (!(best > JR(0))) return false;
        p = bi;
      }
      if (lane == 0) PIV[k] = p;
      if (p != k)
        for (int j = k + lane; j < N; j += 32) {
          const JR tmp = A[k * LDA + j];
          A[k * LDA + j] = A[p * LDA + j];
          A[p * LDA + j] = tmp;
        }
      __syncwarp();
      const JR inv = JR(1) / A[k * LDA + k];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = idx(r);
        if (i > k && i < N) {
          const JR l = A[i * LDA + k] * inv;
          A[i * LDA + k] = l;
#pragma unroll 4
          for (int j = k + 1; j < N; ++j) A[i * LDA + j] -= l * A[k * LDA + j];
        }
      }
      __syncwarp();
      if (lane == 0) A[k * LDA + k] = inv;
      __syncwarp();
    }
    return true;
  };
  jacobian(yv.v);
  if constexpr (FACTOR) return factor(gamma);
  else return true;
}

// (I - gamma J) x = b with the factors warp_setup left in A / PIV (trailing row swaps,
// reciprocal pivots on the diagonal): one warp, rows over lanes, b distributed like the state
// (element i in lane i mod 32) and overwritten with x; XS is the N-element staging vector.
template <class M, class JR>
__device__ __forceinline__ void warp_lu_solve(const JR* A, const int* PIV, JR* XS, double (&b)[(M::N + 31) / 32]) {
  constexpr int N = M::N, R = (N + 31) / 32, LDA = N + 1;
  const int lane = threadIdx.x & 31;
  auto idx = [&](int r) { return lane + 32 * r; };
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (idx(r) < N) XS[idx(r)] = (JR)b[r];
  __syncwarp();
#pragma unroll 1
  for (int k = 0; k < N; ++k) {
    const int p = PIV[k];
    if (p != k && lane == 0) { const JR tmp = XS[k]; XS[k] = XS[p]; XS[p] = tmp; }
    __syncwarp();
    const JR bk = XS[k];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = idx(r);
      if (i > k && i < N) XS[i] -= A[i * LDA + k] * bk;
    }
    __syncwarp();
  }
#pragma unroll 1
  for (int k = N - 1; k >= 0; --k) {
    const JR xk = XS[k] * A[k * LDA + k];
    __syncwarp();
    if (lane == 0) XS[k] = xk;
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = idx(r);
      if (i < k) XS[i] -= A[i * LDA + k] * xk;
    }
    __syncwarp();
  }
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (idx(r) < N) b[r] = (double)XS[idx(r)];
  __syncwarp();
}

template <class M, class JR, int WPB>
__global__ void __launch_bounds__(WPB * 32, 1) bdf_warp_kernel(const ReactParams P) {
  using namespace bdf;
  using Tab = typename M::TabG;
  constexpr int N = M::N, NS = M::NS, NR = M::NR;
  constexpr int R = (N + 31) / 32;   // vector elements per lane
  constexpr int LDA = N + 1;         // padded matrix row
  constexpr bool MIXED = sizeof(JR) == sizeof(float);
  extern __shared__ __align__(16) unsigned char wsmem[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  unsigned char* base = wsmem + (size_t)wid * bdf_warp_smem_per_warp<M, JR>();
  double* Z = reinterpret_cast<double*>(base);   // [(QMAX+2)][N]
  double* FRC = Z + (QMAX + 2) * N;              // [N] forcing (rhoY, then rho h)
  double* LC = FRC + N;                          // [QMAX+1] l coefficients
  double* TAU = LC + (QMAX + 1);                 // [QMAX+2] step history
  unsigned char* const scratch = base + bdf_warp_state_bytes<M>();  // RHS | setup scratch
  double* CS = reinterpret_cast<double*>(scratch);  // [NS] concentrations
  double* GS = CS + NS;                          // [NS] g/RT
  double* QS = GS + NS;                          // [NR] rates of progress
  JR* RX = reinterpret_cast<JR*>(scratch);       // [NR][RXW] Jacobian partials
  JR* TH = RX + wbdf::RXW * NR;                  // [4][NS] NASA-7 terms of the setup
  JR* A = reinterpret_cast<JR*>(scratch + bdf_warp_scratch_bytes<M, JR>());  // [N][LDA] Jacobian, then its LU
  JR* XS = A + N * LDA;                          // [N] solve vector
  int* PIV = reinterpret_cast<int*>(XS + N);

  const long long ncell = P.ncell_dev ? (long long)*P.ncell_dev : P.ncell;
  const int qmax = max(1, min(P.max_order, QMAX));
  const double tout = P.dt;

  // ---- lane-distributed vectors: element i = lane + 32 r ----
  auto idx = [&](int r) { return lane + 32 * r; };
  auto bcast = [&](const double (&v)[R], int i) -> double {
    return __shfl_sync(0xffffffffu, v[i >> 5], i & 31);
  };
  double ewt[R];
  auto wms = [&](const double (&v)[R]) -> double {  // squared WRMS norm
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < N) { const double x = v[r] * ewt[r]; s = fma(x, x, s); }
    return warp_sum(s) * (1.0 / N);
  };

  // ---- right-hand side: f = [W_k wdot_k + F_k, dT/dt] at y ----
  auto rhs = [&](const double (&y)[R], double (&f)[R]) {
    WVec<M> yv;
#pragma unroll
    for (int r = 0; r < R; ++r) yv.v[r] = y[r];
    const WVec<M> fv = warp_rhs<M>(yv, CS, GS, QS, FRC);
#pragma unroll
    for (int r = 0; r < R; ++r) f[r] = fv.v[r];
  };

  // ---- analytic Jacobian into A (equations of jac_table, mech_tables.cuh), in type JR ----
  auto solve = [&](double (&b)[R]) { warp_lu_solve<M, JR>(A, PIV, XS, b); };

  for (;;) {
    // ---------------------------------------------- next cell (work stealing, one per warp)
    unsigned long long cnext = 0;
    if (lane == 0) cnext = atomicAdd(P.next_cell, 1ull);
    cnext = __shfl_sync(0xffffffffu, cnext, 0);
    if ((long long)cnext >= ncell) break;
    const long long cell = P.cell_list ? P.cell_list[cnext] : (long long)cnext;
    int lo = 0, hi = P.nbox - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (P.boxes[mid].cell_offset <= cell) lo = mid; else hi = mid - 1;
    }
    const BoxDev& B = P.boxes[lo];
    long long rr = cell - B.cell_offset;
    const int ci = B.lo0 + (int)(rr % B.len0);
    rr /= B.len0;
    const int cj = B.lo1 + (int)(rr % B.len1);
    const int ck = B.lo2 + (int)(rr / B.len1);
    auto elem = [&](const ArrDev& a, int n) -> double& {
      return a.p[(long long)(ci - a.begin0) + (long long)(cj - a.begin1) * a.jstride +
                 (long long)(ck - a.begin2) * a.kstride + (long long)n * a.nstride];
    };
    if (B.mask.p && B.mask.p[(long long)(ci - B.mask.begin0) + (long long)(cj - B.mask.begin1) * B.mask.jstride +
                             (long long)(ck - B.mask.begin2) * B.mask.kstride] < 0) {
      if (lane == 0) elem(B.FC, 0) = 0.0;
      if (B.IR.p)
        for (int k = lane; k < NS; k += 32) elem(B.IR, k) = -elem(B.rYsrc, k);
      continue;
    }
    double y[R], f[R], acor[R], tmp[R], acor_saved[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = idx(r);
      y[r] = 0.0; f[r] = 0.0; acor[r] = 0.0; tmp[r] = 0.0; acor_saved[r] = 0.0; ewt[r] = 1.0;
      if (i < NS) { y[r] = elem(B.rY, i) * B.sY_in; FRC[i] = elem(B.rYsrc, i) * B.sY_in; }
      else if (i == NS) { y[r] = elem(B.T, 0); FRC[NS] = elem(B.rEsrc, 0) * B.sE_in; }
      if (i < N) Z[i] = y[r];
    }
    const double rE0 = elem(B.rE, 0) * B.sE_in;
    if (lane < QMAX + 2) TAU[lane] = 0.0;
    __syncwarp();
    auto zget = [&](int j, int r) -> double& { return Z[j * N + idx(r)]; };
    auto set_ewt = [&]() {
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (idx(r) < N) {
          const double d = fma(P.rtol, fabs(zget(0, r)), P.atol[idx(r)]);
          ewt[r] = MIXED ? recip_fast(d) : 1.0 / d;
        }
    };

    double t = 0.0, h = 0.0, hscale = 0.0, etamax = ETAMX1, eta = 1.0;
    double gamma = 0.0, gammap = 0.0, gamrat = 1.0, crate2 = 1.0, rl1 = 1.0, acnrm2 = 0.0;
    double tq1 = 1.0, tq2 = 1.0, tq3 = 1.0, tq5 = 1.0, tq5_saved = 1.0, inv_tq4_sq = 1.0;
    int q = 1, qwait = 2, nef = 0, ncf = 0, status = OK;
    long long nst = 0, nfe = 0, nje = 0, nstlp = 0, netf = 0, ncfn = 0;
    bool force_setup = true;

    auto rescale = [&](double e) {
      double fac = e;
      for (int j = 1; j <= q; ++j) {
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (idx(r) < N) zget(j, r) *= fac;
        fac *= e;
      }
      h = hscale * e;
      hscale = h;
    };
    auto predict = [&]() {
      t += h;
      for (int k = 1; k <= q; ++k)
        for (int j = q; j >= k; --j)
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (idx(r) < N) zget(j - 1, r) += zget(j, r);
    };
    auto retract = [&]() {
      t -= h;
      for (int k = 1; k <= q; ++k)
        for (int j = q; j >= k; --j)
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (idx(r) < N) zget(j - 1, r) -= zget(j, r);
    };
    // l coefficients and error constants (scalar, every lane; the same arithmetic as the
    // per-thread kernel's set_coeffs)
    auto set_coeffs = [&]() {
      double l[QMAX + 1];
#pragma unroll
      for (int i = 0; i <= QMAX; ++i) l[i] = 0.0;
      l[0] = 1.0;
      double alpha0 = 0.0;
      for (int j = 1; j <= q; ++j) alpha0 -= inv_int(j);
      double hsum = h, sum_xi_inv = 0.0;
      for (int i = 1; i <= q - 1; ++i) {
        if (i > 1) hsum += TAU[i - 1];
        const double xi_inv = h / hsum;
        sum_xi_inv += xi_inv;
#pragma unroll
        for (int k = QMAX; k >= 1; --k)
          if (k <= i) l[k] += l[k - 1] * xi_inv;
      }
      const double xistar_inv = -alpha0 - sum_xi_inv;
#pragma unroll
      for (int k = QMAX; k >= 1; --k)
        if (k <= q) l[k] += l[k - 1] * xistar_inv;
      if (q > 1) hsum += TAU[q - 1];
      const double xiq_inv = h / hsum;
      const double alpha0_hat = -(sum_xi_inv + xiq_inv);
      const double A1 = 1.0 - alpha0_hat + alpha0;
      const double A2 = 1.0 + q * A1;
      double lq = 0.0;
#pragma unroll
      for (int k = 0; k <= QMAX; ++k) if (k == q) lq = l[k];
      tq2 = fabs(A1 / (alpha0 * A2));
      tq5 = fabs(A2 * xistar_inv / (lq * xiq_inv));
      if (qwait == 1) {
        if (q > 1) {
          const double C = xistar_inv / lq;
          const double A3 = alpha0 + inv_int(q);
          const double A4 = alpha0_hat + xiq_inv;
          tq1 = fabs(C * (1.0 - A4 + A3) / A3);
        } else {
          tq1 = 1.0;
        }
        const double xiq1_inv = h / (hsum + TAU[q]);
        const double A5 = alpha0 - inv_int(q + 1);
        const double A6 = alpha0_hat - xiq1_inv;
        const double Cpp = (1.0 - A6 + A5) / A2;
        tq3 = fabs(Cpp / (xiq1_inv * (q + 2) * A5));
      }
      inv_tq4_sq = (tq2 * (1.0 / NLSCOEF)) * (tq2 * (1.0 / NLSCOEF));
      __syncwarp();
      if (lane <= QMAX) {
        double v = 0.0;
#pragma unroll
        for (int k = 0; k <= QMAX; ++k) if (k == lane) v = l[k];
        LC[lane] = v;
      }
      __syncwarp();
    };
    auto adjust_order = [&](int dq) {
      double w[QMAX + 2];
#pragma unroll
      for (int i = 0; i < QMAX + 2; ++i) w[i] = 0.0;
      w[2] = 1.0;
      if (dq > 0) {
        double alpha0 = 0.0, alpha1 = 0.0, prod = 1.0, hsum = 0.0;
        for (int j = 1; j <= q; ++j) {
          hsum += TAU[j];
          const double xi = hsum / hscale;
          prod *= xi;
          alpha0 -= inv_int(j);
          alpha1 += 1.0 / xi;
          if (j <= q - 1)
#pragma unroll
            for (int i = QMAX + 1; i >= 2; --i)
              if (i <= j + 2) w[i] = w[i] * xi + w[i - 1];
        }
        const double A1 = (-alpha0 - alpha1) / prod;
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (idx(r) < N) zget(q + 1, r) = A1 * acor_saved[r];
#pragma unroll
        for (int j = 2; j <= QMAX; ++j)
          if (j <= q)
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (idx(r) < N) zget(j, r) = fma(w[j], zget(q + 1, r), zget(j, r));
      } else {
        double hsum = 0.0;
        for (int j = 1; j <= q - 2; ++j) {
          hsum += TAU[j];
          const double xi = hsum / hscale;
#pragma unroll
          for (int i = QMAX + 1; i >= 2; --i)
            if (i <= j + 2) w[i] = w[i] * xi + w[i - 1];
        }
#pragma unroll
        for (int j = 2; j <= QMAX; ++j)
          if (j < q)
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (idx(r) < N) zget(j, r) = fma(-w[j], zget(q, r), zget(j, r));
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (idx(r) < N) zget(q, r) = 0.0;
      }
    };
    // modified Newton on the corrector; 0 converged, 1 convergence failure, 2 singular matrix
    auto newton = [&]() -> int {
      bool call_setup = force_setup || nst == 0 || nst >= nstlp + MSBP || fabs(gamrat - 1.0) > DGMAX;
      force_setup = false;
      for (;;) {
#pragma unroll
        for (int r = 0; r < R; ++r) { y[r] = idx(r) < N ? zget(0, r) : 0.0; acor[r] = 0.0; }
        rhs(y, f);
        ++nfe;
        bool jcur = false;
        if (call_setup) {
          WVec<M> yv;
#pragma unroll
          for (int r = 0; r < R; ++r) yv.v[r] = y[r];
          ++nje;
          const bool ok = warp_setup<M, JR>(yv, gamma, FRC, A, XS, RX, TH, PIV);
          gammap = gamma;
          gamrat = 1.0;
          crate2 = 1.0;
          nstlp = nst;
          if (!ok) return 2;
          jcur = true;
          call_setup = false;
        }
        double delp2 = 0.0, del2 = 0.0;
        int mm = 0;
        bool ok = false;
        for (;;) {
#pragma unroll
          for (int r = 0; r < R; ++r)
            tmp[r] = idx(r) < N ? fma(gamma, f[r], -fma(rl1, zget(1, r), acor[r])) : 0.0;
          solve(tmp);
          if (gamrat != 1.0) {
            const double s = 2.0 / (1.0 + gamrat);
#pragma unroll
            for (int r = 0; r < R; ++r) tmp[r] *= s;
          }
          del2 = wms(tmp);
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (idx(r) < N) { acor[r] += tmp[r]; y[r] = zget(0, r) + acor[r]; }
          if (mm > 0) crate2 = fmax((CRDOWN * CRDOWN) * crate2, del2 / delp2);
          if (del2 * fmin(1.0, crate2) * inv_tq4_sq <= 1.0) {
            acnrm2 = (mm == 0) ? del2 : wms(acor);
            ok = true;
            break;
          }
          ++mm;
          if (mm == MAXCOR || (mm >= 2 && del2 > (RDIV * RDIV) * delp2)) break;
          delp2 = del2;
          rhs(y, f);
          ++nfe;
          if (!isfinite(bcast(f, 0))) break;
        }
        if (ok) return 0;
        if (!jcur) { call_setup = true; continue; }
        return 1;
      }
    };

    // ---------------------------------------------- initial step size
    rhs(y, f);
    ++nfe;
    set_ewt();
    {
      const double tround = UROUND * tout;
      const double hlb = 100.0 * tround;
      double hub_inv = 0.0;
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (idx(r) < N) hub_inv = fmax(hub_inv, fabs(f[r]) / fma(0.1, fabs(zget(0, r)), P.atol[idx(r)]));
      hub_inv = warp_max(hub_inv);
      double hub = 0.1 * tout;
      if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
      double hg = sqrt(hlb * hub), hnew = hg;
      if (hub > hlb) {
        for (int count = 1; count <= 4; ++count) {
          double yy[R], fy[R];
#pragma unroll
          for (int r = 0; r < R; ++r) yy[r] = idx(r) < N ? fma(hg, f[r], zget(0, r)) : 0.0;
          rhs(yy, fy);
          ++nfe;
#pragma unroll
          for (int r = 0; r < R; ++r) tmp[r] = (fy[r] - f[r]) / hg;
          const double ydd = sqrt(wms(tmp));
          hnew = (ydd * hub * hub > 2.0) ? sqrt(2.0 / ydd) : sqrt(hg * hub);
          if (count == 4) break;
          const double hrat = hnew / hg;
          if (hrat > 0.5 && hrat < 2.0) break;
          if (count >= 2 && hrat > 2.0) { hnew = hg; break; }
          hg = hnew;
        }
      }
      h = fmin(fmax(0.5 * hnew, hlb), hub);
    }
    hscale = h;
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < N) zget(1, r) = h * f[r];
    q = 1; qwait = 2; etamax = ETAMX1;
    if (lane == 0) TAU[1] = h;
    __syncwarp();

    // ---------------------------------------------- step loop
    for (;;) {
      if (nst >= P.max_steps) { status = MAX_STEPS; break; }
      if ((t + h - tout) * h > 0.0) rescale((tout - t) * (1.0 - 4.0 * UROUND) / h);
      set_ewt();
      nef = 0; ncf = 0;
      double dsm2 = 0.0;
      bool failed = false;
      for (;;) {
        predict();
        set_coeffs();
        rl1 = 1.0 / LC[1];
        gamma = h * rl1;
        if (nst == 0) gammap = gamma;
        gamrat = (nst > 0) ? gamma / gammap : 1.0;
        const int nflag = newton();
        if (nflag != 0) {
          retract();
          ++ncf; ++ncfn;
          if (nflag == 2 || ncf >= MXNCF || fabs(h) <= 100.0 * UROUND * fabs(t)) { status = CONV; failed = true; break; }
          force_setup = true;
          etamax = 1.0;
          rescale(ETACF);
          continue;
        }
        dsm2 = acnrm2 * (tq2 * tq2);
        if (!(dsm2 <= 1.0)) {
          retract();
          ++nef; ++netf;
          if (nef >= MXNEF || !isfinite(dsm2)) { status = isfinite(dsm2) ? ERRTEST : NONFINITE; failed = true; break; }
          etamax = 1.0;
          if (nef <= MXNEF1) {
            double e = 1.0 / (pgb_pow64((BIAS2 * BIAS2) * dsm2, 0.5 * inv_int(q + 1)) + ADDON);
            e = fmax(ETAMIN, e);
            if (nef >= SMALL_NEF) e = fmin(e, ETAMXF);
            rescale(e);
          } else if (q > 1) {
            adjust_order(-1);
            --q;
            qwait = q + 1;
            rescale(ETAMIN);
          } else {
            rescale(ETAMIN);
#pragma unroll
            for (int r = 0; r < R; ++r) y[r] = idx(r) < N ? zget(0, r) : 0.0;
            rhs(y, f);
            ++nfe;
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (idx(r) < N) zget(1, r) = h * f[r];
            qwait = 10;
          }
          if (fabs(h) <= 100.0 * UROUND * fabs(t)) { status = HSMALL; failed = true; break; }
          continue;
        }
        break;
      }
      if (failed) break;
      // ---- complete the step ----
      ++nst;
      __syncwarp();
      if (lane == 0) {
        for (int i = q + 1; i >= 2; --i) TAU[i] = TAU[i - 1];
        TAU[1] = h;
      }
      for (int j = 0; j <= q; ++j) {
        const double lj = LC[j];
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (idx(r) < N) zget(j, r) = fma(lj, acor[r], zget(j, r));
      }
      __syncwarp();
      --qwait;
      if (qwait == 1 && q != qmax) {
#pragma unroll
        for (int r = 0; r < R; ++r) acor_saved[r] = acor[r];
        tq5_saved = tq5;
      }
      if (fabs(t - tout) <= 100.0 * UROUND * (fabs(t) + fabs(h)) || t >= tout) break;
      // ---- next step size and order ----
      const double etaq = 1.0 / (pgb_pow64((BIAS2 * BIAS2) * dsm2, 0.5 * inv_int(q + 1)) + ADDON);
      int qprime = q;
      if (etamax == 1.0) {
        qwait = max(qwait, 2);
        eta = 1.0;
      } else {
        eta = etaq;
        if (qwait == 0) {
          qwait = 2;
          double etaqm1 = 0.0, etaqp1 = 0.0;
          if (q > 1) {
            double zq[R];
#pragma unroll
            for (int r = 0; r < R; ++r) zq[r] = idx(r) < N ? zget(q, r) : 0.0;
            const double ddn2 = wms(zq) * (tq1 * tq1);
            etaqm1 = 1.0 / (pgb_pow64((BIAS1 * BIAS1) * ddn2, 0.5 * inv_int(q)) + ADDON);
          }
          if (q != qmax) {
            const double hr = h / TAU[2];
            double hrp = hr;
            for (int k = 0; k < q; ++k) hrp *= hr;
            const double cquot = (tq5 / tq5_saved) * hrp;
#pragma unroll
            for (int r = 0; r < R; ++r) tmp[r] = acor[r] - cquot * acor_saved[r];
            const double dup2 = wms(tmp) * (tq3 * tq3);
            etaqp1 = 1.0 / (pgb_pow64((BIAS3 * BIAS3) * dup2, 0.5 * inv_int(q + 2)) + ADDON);
          }
          const double etam = fmax(etaqm1, fmax(etaq, etaqp1));
          if (etam < THRESH) {
            eta = 1.0;
          } else if (etam == etaq) {
            eta = etaq;
          } else if (etam == etaqm1) {
            eta = etaqm1;
            qprime = q - 1;
          } else {
            eta = etaqp1;
            qprime = q + 1;
#pragma unroll
            for (int r = 0; r < R; ++r) acor_saved[r] = acor[r];
          }
        } else if (eta < THRESH) {
          eta = 1.0;
        }
        if (eta >= THRESH || qprime != q) eta = fmin(eta, etamax);
        else eta = 1.0;
      }
      etamax = (nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
      if (qprime != q) {
        adjust_order(qprime - q);
        q = qprime;
        qwait = q + 1;
      }
      if (eta != 1.0) rescale(eta);
      __syncwarp();
    }

    // ---------------------------------------------- finish: rho h(t), T from (h, Y)
    __syncwarp();
    if (status != OK && P.retry_list) {  // hand the cell to the retry pass, arrays untouched
      if (lane == 0) {
        P.retry_list[atomicAdd(P.retry_count, 1ull)] = cell;
        ReactStats* S = P.stats;
        atomicAdd(&S->nst, (unsigned long long)nst);
        atomicAdd(&S->nfe, (unsigned long long)nfe);
        atomicAdd(&S->nje, (unsigned long long)nje);
        atomicAdd(&S->netf, (unsigned long long)netf);
        atomicAdd(&S->ncfn, (unsigned long long)ncfn);
        atomicAdd(&S->nretry, 1ull);
      }
      __syncwarp();
      continue;
    }
    const double rE = fma(tout, FRC[NS], rE0);
    double rho_l = 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < NS) rho_l += zget(0, r);
    const double inv_rho = 1.0 / warp_sum(rho_l);
    const double htarget = rE * inv_rho;
    double Tn = Z[NS];
    if (!(Tn > 90.0 && Tn < 5000.0)) Tn = 1000.0;
    for (int it = 0; it < 50; ++it) {
      double hl = 0.0, cl = 0.0;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int k = idx(r);
        if (k < NS) {
          const TabSpecies<double>& s = Tab::template sp<double>(k);
          const bool lo = Tn < s.Tmid;
          const double* a = lo ? s.lo : s.hi;
          const double* hc = lo ? s.hlo : s.hhi;
          const double invTn = 1.0 / Tn;
          const double hRT = fma(Tn, fma(Tn, fma(Tn, fma(Tn, hc[4], hc[3]), hc[2]), hc[1]), fma(hc[5], invTn, hc[0]));
          const double cpR = fma(Tn, fma(Tn, fma(Tn, fma(Tn, a[4], a[3]), a[2]), a[1]), a[0]);
          const double Yk = zget(0, r) * inv_rho;
          hl = fma(Yk * s.invW, hRT * kRerg * Tn, hl);
          cl = fma(Yk * s.invW, cpR * kRerg, cl);
        }
      }
      const double hh = warp_sum(hl), cp = warp_sum(cl);
      double dT = (htarget - hh) / cp;
      dT = fmax(-100.0, fmin(100.0, dT));
      Tn = fmax(90.0, fmin(5000.0, Tn + dT));
      if (fabs(dT) < 1e-10 * Tn) break;
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < NS) {
        const double rYn = __dmul_rn(zget(0, r), B.sY_out);
        if (B.IR.p)  // separate roundings, as separate passes over arrays give
          elem(B.IR, idx(r)) = __dsub_rn(__dmul_rn(-__dsub_rn(elem(B.rY, idx(r)), rYn), 1.0 / tout),
                                         elem(B.rYsrc, idx(r)));
        elem(B.rY, idx(r)) = rYn;
      }
    if (lane == 0) {
      elem(B.T, 0) = Tn;
      elem(B.rE, 0) = rE * B.sE_out;
      elem(B.FC, 0) = (status == OK) ? (double)nfe : -(double)status;
      ReactStats* S = P.stats;
      atomicAdd(&S->nst, (unsigned long long)nst);
      atomicAdd(&S->nfe, (unsigned long long)nfe);
      atomicAdd(&S->nje, (unsigned long long)nje);
      atomicAdd(&S->netf, (unsigned long long)netf);
      atomicAdd(&S->ncfn, (unsigned long long)ncfn);
      if (status != OK) atomicAdd(&S->nfail, 1ull);
      atomicMax(&S->max_nst, (unsigned long long)nst);
      const int bin = min(15, 31 - __clz((int)max(nst, 1LL)));
      atomicAdd(&S->hist[bin], 1ull);
    }
    __syncwarp();
  }
}

}  // namespace pgb

#endif  // PGB_BDF_WARP_KERNEL_CUH
