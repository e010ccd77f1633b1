// CPU oracle: thermo, kinetics, reactor RHS, analytic Jacobian and T(h) — table-driven.
// TEST INFRASTRUCTURE ONLY (see chem_oracle.hpp for scope and parity status).
//
// The RHS is written once as a template on the scalar type so the same code runs in
// double (the oracle / CPU baseline) and with a counting scalar (algorithmic FP64 op
// count of one RHS evaluation).
#include "chem_oracle.hpp"

#include <algorithm>
#include <fstream>
#include <sstream>

namespace orc {

bool Mechanism::load(const std::string& path, std::string* err) {
  std::ifstream f(path);
  if (!f) {
    if (err) *err = "cannot open " + path;
    return false;
  }
  f >> ns >> nr >> nel;
  if (!f || ns <= 0 || ns > MAXNS || nr < 0 || nr > MAXNR) {
    if (err) *err = "bad header in " + path;
    return false;
  }
  W.resize(ns); Tmid.resize(ns); lo.resize(ns); hi.resize(ns); comp.resize(ns);
  for (int k = 0; k < ns; ++k) {
    f >> W[k] >> Tmid[k];
    for (int i = 0; i < 7; ++i) f >> lo[k][i];
    for (int i = 0; i < 7; ++i) f >> hi[k][i];
    int nc; f >> nc;
    for (int i = 0; i < nc; ++i) { int e, n; f >> e >> n; comp[k].push_back({e, n}); }
  }
  rx.resize(nr);
  for (int j = 0; j < nr; ++j) {
    Reaction& r = rx[j];
    int rev; f >> r.kind >> rev; r.reversible = rev != 0;
    int n; f >> n;
    for (int i = 0; i < n; ++i) { int s, nu; f >> s >> nu; r.reac.push_back({s, nu}); }
    f >> n;
    for (int i = 0; i < n; ++i) { int s, nu; f >> s >> nu; r.prod.push_back({s, nu}); }
    f >> r.A >> r.beta >> r.Ea;
    if (r.kind == 2) {
      f >> r.A0 >> r.beta0 >> r.Ea0;
      int nt; f >> nt; r.troe.resize(nt);
      for (int i = 0; i < nt; ++i) f >> r.troe[i];
    }
    if (r.kind >= 1) {
      int ne; f >> ne;
      for (int i = 0; i < ne; ++i) { int s; double e; f >> s >> e; r.eff.push_back({s, e}); }
    }
    r.lnA = std::log(r.A);
    r.lnA0 = (r.kind == 2) ? std::log(r.A0) : 0.0;
    r.dnu = 0;
    for (auto& sn : r.prod) r.dnu += sn.second;
    for (auto& sn : r.reac) r.dnu -= sn.second;
  }
  if (!f) {
    if (err) *err = "parse error in " + path;
    return false;
  }
  return true;
}

// ------------------------------------------------------------------ templated core
template <class R>
struct Core {
  // per-species cp/R, h/RT, g/RT at T (lnT given)
  static void thermo(const Mechanism& m, R T, R lnT, R* cpR, R* hRT, R* gRT) {
    const R T2 = T * T, T3 = T2 * T, T4 = T3 * T, invT = R(1.0) / T;
    for (int k = 0; k < m.ns; ++k) {
      const auto& a = (value(T) < m.Tmid[k]) ? m.lo[k] : m.hi[k];
      if (cpR) cpR[k] = a[0] + a[1] * T + a[2] * T2 + a[3] * T3 + a[4] * T4;
      const R h = a[0] + a[1] * 0.5 * T + a[2] * (1.0 / 3.0) * T2 + a[3] * 0.25 * T3 +
                  a[4] * 0.2 * T4 + a[5] * invT;
      if (hRT) hRT[k] = h;
      if (gRT) {
        const R s = a[0] * lnT + a[1] * T + a[2] * 0.5 * T2 + a[3] * (1.0 / 3.0) * T3 +
                    a[4] * 0.25 * T4 + a[6];
        gRT[k] = h - s;
      }
    }
  }

  // rate of progress of every reaction and the falloff / T-derivative data the Jacobian needs
  struct RxData {
    R kf, kr, alpha, Pf, Pr, q, dlnkf, dlnkr, dkeff_dM;
  };

  static void reactions(const Mechanism& m, R T, R lnT, const R* C, const R* gRT,
                        const R* hRT, RxData* out, bool need_derivs) {
    using std::exp;
    using std::log;
    using std::log10;
    using std::pow;
    const R invT = R(1.0) / T;
    const R invRcT = invT * (1.0 / R_CAL);
    const R lnP0RT = log(R(P_ATM / R_ERG) * invT);
    R Ctot = R(0.0);
    for (int k = 0; k < m.ns; ++k) Ctot = Ctot + C[k];
    for (int j = 0; j < m.nr; ++j) {
      const Reaction& r = m.rx[j];
      RxData& e = out[j];
      R kf = exp(r.lnA + r.beta * lnT - r.Ea * invRcT);
      R dlnkf = R(0.0);
      if (need_derivs) dlnkf = (r.beta + r.Ea * invRcT) * invT;
      R M = R(0.0);
      if (r.kind >= 1) {
        M = Ctot;
        for (auto& se : r.eff) M = M + (se.second - 1.0) * C[se.first];
      }
      e.alpha = R(1.0);
      e.dkeff_dM = R(0.0);
      if (r.kind == 1) {
        e.alpha = M;
      } else if (r.kind == 2) {
        const R k0 = exp(r.lnA0 + r.beta0 * lnT - r.Ea0 * invRcT);
        const R Pr = k0 * M / kf;
        R F = R(1.0);
        if (!r.troe.empty()) {
          const double a = r.troe[0];
          R Fcent = (1.0 - a) * exp(-T / r.troe[1]) + a * exp(-T / r.troe[2]);
          if (r.troe.size() > 3) Fcent = Fcent + exp(R(-r.troe[3]) * invT);
          const R lFc = log10(Fcent);
          const R c = -0.4 - 0.67 * lFc, n = 0.75 - 1.27 * lFc;
          const R lPr = log10(value(Pr) > 1e-300 ? Pr : R(1e-300));
          const R f1 = (lPr + c) / (n - 0.14 * (lPr + c));
          F = pow(R(10.0), lFc / (1.0 + f1 * f1));
        }
        const R kinf = kf;
        const R onePr = R(1.0) + Pr;
        kf = kinf * Pr / onePr * F;
        if (need_derivs) {
          e.dkeff_dM = F * k0 / (onePr * onePr);
          const R dlnk0 = (r.beta0 + r.Ea0 * invRcT) * invT;
          dlnkf = dlnkf + (dlnk0 - dlnkf) / onePr;
        }
      }
      e.kf = kf;
      e.dlnkf = dlnkf;
      e.kr = R(0.0);
      e.dlnkr = R(0.0);
      if (r.reversible) {
        R dG = R(0.0), dH = R(0.0);
        for (auto& sn : r.prod) {
          dG = dG + sn.second * gRT[sn.first];
          if (need_derivs) dH = dH + sn.second * hRT[sn.first];
        }
        for (auto& sn : r.reac) {
          dG = dG - sn.second * gRT[sn.first];
          if (need_derivs) dH = dH - sn.second * hRT[sn.first];
        }
        // kr = kf / Kc,  Kc = exp(-dG) (P0/RT)^dnu. The exponent is capped at 700 (exp stays
        // finite): far below equilibrium at low T it overflows, and inf times an absent
        // product's zero concentration would turn the rate of progress into NaN.
        R arg = dG - r.dnu * lnP0RT;
        if (value(arg) > 700.0) arg = R(700.0);
        e.kr = kf * exp(arg);
        if (need_derivs) e.dlnkr = dlnkf - (dH - r.dnu) * invT;
      }
      R Pf = R(1.0), Pp = R(1.0);
      for (auto& sn : r.reac)
        for (int i = 0; i < sn.second; ++i) Pf = Pf * C[sn.first];
      for (auto& sn : r.prod)
        for (int i = 0; i < sn.second; ++i) Pp = Pp * C[sn.first];
      e.Pf = Pf;
      e.Pr = Pp;
      e.q = e.alpha * (e.kf * Pf - e.kr * Pp);
    }
  }

  static void rhs(const Mechanism& m, const R* y, const R* Fsrc, R Fh, R* ydot) {
    using std::log;
    const int ns = m.ns;
    const R T = y[ns];
    const R lnT = log(T);
    R C[MAXNS], cpR[MAXNS], hRT[MAXNS], gRT[MAXNS], wdot[MAXNS];
    for (int k = 0; k < ns; ++k) { C[k] = y[k] * (1.0 / m.W[k]); wdot[k] = R(0.0); }
    thermo(m, T, lnT, cpR, hRT, gRT);
    RxData rd[MAXNR];
    reactions(m, T, lnT, C, gRT, hRT, rd, false);
    for (int j = 0; j < m.nr; ++j) {
      const Reaction& r = m.rx[j];
      for (auto& sn : r.reac) wdot[sn.first] = wdot[sn.first] - sn.second * rd[j].q;
      for (auto& sn : r.prod) wdot[sn.first] = wdot[sn.first] + sn.second * rd[j].q;
    }
    R rcp = R(0.0), hsum = R(0.0);
    const R RT = R_ERG * T;
    for (int k = 0; k < ns; ++k) {
      const R wm = wdot[k] * m.W[k] + Fsrc[k];
      ydot[k] = wm;
      rcp = rcp + y[k] * cpR[k] * (R_ERG / m.W[k]);
      hsum = hsum + hRT[k] * (1.0 / m.W[k]) * wm;
    }
    ydot[ns] = (Fh - hsum * RT) / rcp;
  }

  static double value(const R& x);
};

template <>
double Core<double>::value(const double& x) { return x; }

// ------------------------------------------------------------------ counting scalar
namespace counting {
struct Cnt {
  double v;
  Cnt(double x = 0.0) : v(x) {}
};
thread_local long g_ops = 0, g_trans = 0;
inline Cnt operator+(Cnt a, Cnt b) { ++g_ops; return Cnt(a.v + b.v); }
inline Cnt operator-(Cnt a, Cnt b) { ++g_ops; return Cnt(a.v - b.v); }
inline Cnt operator*(Cnt a, Cnt b) { ++g_ops; return Cnt(a.v * b.v); }
inline Cnt operator/(Cnt a, Cnt b) { ++g_ops; return Cnt(a.v / b.v); }
inline Cnt operator-(Cnt a) { return Cnt(-a.v); }
inline Cnt operator+(double a, Cnt b) { return Cnt(a) + b; }
inline Cnt operator-(double a, Cnt b) { return Cnt(a) - b; }
inline Cnt operator*(double a, Cnt b) { return Cnt(a) * b; }
inline Cnt operator/(double a, Cnt b) { return Cnt(a) / b; }
inline Cnt operator+(Cnt a, double b) { return a + Cnt(b); }
inline Cnt operator-(Cnt a, double b) { return a - Cnt(b); }
inline Cnt operator*(Cnt a, double b) { return a * Cnt(b); }
inline Cnt operator/(Cnt a, double b) { return a / Cnt(b); }
inline Cnt operator*(int a, Cnt b) { return Cnt(double(a)) * b; }
inline Cnt exp(Cnt a) { ++g_trans; return Cnt(std::exp(a.v)); }
inline Cnt log(Cnt a) { ++g_trans; return Cnt(std::log(a.v)); }
inline Cnt log10(Cnt a) { ++g_trans; return Cnt(std::log10(a.v)); }
inline Cnt pow(Cnt a, Cnt b) { ++g_trans; return Cnt(std::pow(a.v, b.v)); }
}  // namespace counting

template <>
double Core<counting::Cnt>::value(const counting::Cnt& x) { return x.v; }

// ------------------------------------------------------------------ public (double)
void species_thermo(const Mechanism& m, int k, double T, double* cpR, double* hRT, double* sR,
                    double* dcpRdT) {
  const auto& a = (T < m.Tmid[k]) ? m.lo[k] : m.hi[k];
  const double T2 = T * T, T3 = T2 * T, T4 = T3 * T;
  if (cpR) *cpR = a[0] + a[1] * T + a[2] * T2 + a[3] * T3 + a[4] * T4;
  if (hRT) *hRT = a[0] + a[1] * T / 2 + a[2] * T2 / 3 + a[3] * T3 / 4 + a[4] * T4 / 5 + a[5] / T;
  if (sR) *sR = a[0] * std::log(T) + a[1] * T + a[2] * T2 / 2 + a[3] * T3 / 3 + a[4] * T4 / 4 + a[6];
  if (dcpRdT) *dcpRdT = a[1] + 2 * a[2] * T + 3 * a[3] * T2 + 4 * a[4] * T3;
}

void production_rates(const Mechanism& m, double T, const double* C, double* wdot) {
  double hRT[MAXNS], gRT[MAXNS];
  const double lnT = std::log(T);
  Core<double>::thermo(m, T, lnT, nullptr, hRT, gRT);
  Core<double>::RxData rd[MAXNR];
  Core<double>::reactions(m, T, lnT, C, gRT, hRT, rd, false);
  for (int k = 0; k < m.ns; ++k) wdot[k] = 0.0;
  for (int j = 0; j < m.nr; ++j) {
    const Reaction& r = m.rx[j];
    for (auto& sn : r.reac) wdot[sn.first] -= sn.second * rd[j].q;
    for (auto& sn : r.prod) wdot[sn.first] += sn.second * rd[j].q;
  }
}

void reactor_rhs(const Mechanism& m, const double* y, const double* F, double Fh, double* ydot) {
  Core<double>::rhs(m, y, F, Fh, ydot);
}

void count_rhs_ops(const Mechanism& m, const double* y, const double* F, double Fh, long* ops,
                   long* trans) {
  using counting::Cnt;
  Cnt yc[MAXNS + 1], Fc[MAXNS], out[MAXNS + 1];
  for (int i = 0; i <= m.ns; ++i) yc[i] = Cnt(y[i]);
  for (int i = 0; i < m.ns; ++i) Fc[i] = Cnt(F[i]);
  counting::g_ops = 0;
  counting::g_trans = 0;
  Core<Cnt>::rhs(m, yc, Fc, Cnt(Fh), out);
  *ops = counting::g_ops;
  *trans = counting::g_trans;
}

void reactor_jac(const Mechanism& m, const double* y, const double* F, double Fh, double* J) {
  const int ns = m.ns, N = ns + 1;
  const double T = y[ns], lnT = std::log(T);
  double C[MAXNS], cpR[MAXNS], hRT[MAXNS], gRT[MAXNS];
  for (int k = 0; k < ns; ++k) C[k] = y[k] / m.W[k];
  Core<double>::thermo(m, T, lnT, cpR, hRT, gRT);
  static thread_local Core<double>::RxData rd[MAXNR];
  Core<double>::reactions(m, T, lnT, C, gRT, hRT, rd, true);
  // dW[i][k] = d wdot_i / d C_k (molar), dWdT[i]
  static thread_local double dW[MAXNS * MAXNS];
  double dWdT[MAXNS], wdot[MAXNS], dq[MAXNS];
  for (int i = 0; i < ns * ns; ++i) dW[i] = 0.0;
  for (int k = 0; k < ns; ++k) { dWdT[k] = 0.0; wdot[k] = 0.0; }
  for (int j = 0; j < m.nr; ++j) {
    const Reaction& r = m.rx[j];
    const auto& e = rd[j];
    for (int k = 0; k < ns; ++k) dq[k] = 0.0;
    // mass-action partials: d(P)/dC_k = nu_k C_k^(nu_k-1) prod_{others}
    auto add_partials = [&](const std::vector<std::pair<int, int>>& side, double coef) {
      for (size_t a = 0; a < side.size(); ++a) {
        const int k = side[a].first, nu = side[a].second;
        double p = coef * nu;
        for (int i = 0; i < nu - 1; ++i) p *= C[k];
        for (size_t b = 0; b < side.size(); ++b) {
          if (b == a) continue;
          for (int i = 0; i < side[b].second; ++i) p *= C[side[b].first];
        }
        dq[k] += p;
      }
    };
    add_partials(r.reac, e.alpha * e.kf);
    if (r.reversible) add_partials(r.prod, -e.alpha * e.kr);
    double base = 0.0;
    if (r.kind == 1) {
      base = e.kf * e.Pf - e.kr * e.Pr;
    } else if (r.kind == 2) {
      // kf and kr share the falloff factor: d q / d[M] = dkeff_dM (Pf - Pr / Kc)
      const double inv_Kc = (e.kf != 0.0) ? e.kr / e.kf : 0.0;
      base = e.dkeff_dM * (e.Pf - inv_Kc * e.Pr);
    }
    if (r.kind >= 1) {
      for (int k = 0; k < ns; ++k) dq[k] += base;
      for (auto& se : r.eff) dq[se.first] += (se.second - 1.0) * base;
    }
    const double dqdT = e.alpha * (e.kf * e.dlnkf * e.Pf - e.kr * e.dlnkr * e.Pr);
    for (auto& sn : r.reac) {
      wdot[sn.first] -= sn.second * e.q;
      dWdT[sn.first] -= sn.second * dqdT;
      for (int k = 0; k < ns; ++k) dW[sn.first * ns + k] -= sn.second * dq[k];
    }
    for (auto& sn : r.prod) {
      wdot[sn.first] += sn.second * e.q;
      dWdT[sn.first] += sn.second * dqdT;
      for (int k = 0; k < ns; ++k) dW[sn.first * ns + k] += sn.second * dq[k];
    }
  }
  double cpm[MAXNS], hm[MAXNS], dcpm[MAXNS];
  double D = 0.0, dDdT = 0.0, Q = Fh;
  for (int k = 0; k < ns; ++k) {
    double dcp;
    species_thermo(m, k, T, nullptr, nullptr, nullptr, &dcp);
    cpm[k] = cpR[k] * R_ERG / m.W[k];
    hm[k] = hRT[k] * R_ERG * T / m.W[k];
    dcpm[k] = dcp * R_ERG / m.W[k];
    D += y[k] * cpm[k];
    dDdT += y[k] * dcpm[k];
    Q -= hm[k] * (wdot[k] * m.W[k] + F[k]);
  }
  for (int i = 0; i < ns; ++i) {
    for (int k = 0; k < ns; ++k) J[i * N + k] = m.W[i] * dW[i * ns + k] / m.W[k];
    J[i * N + ns] = m.W[i] * dWdT[i];
  }
  for (int k = 0; k < ns; ++k) {
    double dQ = 0.0;
    for (int i = 0; i < ns; ++i) dQ -= hm[i] * J[i * N + k];
    J[ns * N + k] = dQ / D - Q * cpm[k] / (D * D);
  }
  double dQdT = 0.0;
  for (int i = 0; i < ns; ++i) dQdT -= cpm[i] * (wdot[i] * m.W[i] + F[i]) + hm[i] * J[i * N + ns];
  J[ns * N + ns] = dQdT / D - Q * dDdT / (D * D);
}

double mixture_h(const Mechanism& m, double T, const double* Y) {
  double h = 0.0;
  for (int k = 0; k < m.ns; ++k) {
    double hRT;
    species_thermo(m, k, T, nullptr, &hRT, nullptr, nullptr);
    h += Y[k] * hRT * R_ERG * T / m.W[k];
  }
  return h;
}

int hy2t(const Mechanism& m, double h, const double* Y, double* T) {
  // Newton on h(T) = h_target (cf. Source/PeleLM_K.H:508-529), step limited to 100 K,
  // T clipped to [90, 5000] K
  double t = *T;
  if (!(t > 90.0 && t < 5000.0)) t = 1000.0;
  for (int it = 1; it <= 50; ++it) {
    double hh = 0.0, cp = 0.0;
    for (int k = 0; k < m.ns; ++k) {
      double cpR, hRT;
      species_thermo(m, k, t, &cpR, &hRT, nullptr, nullptr);
      hh += Y[k] * hRT * R_ERG * t / m.W[k];
      cp += Y[k] * cpR * R_ERG / m.W[k];
    }
    double dT = (h - hh) / cp;
    dT = std::max(-100.0, std::min(100.0, dT));
    t = std::max(90.0, std::min(5000.0, t + dT));
    if (std::fabs(dT) < 1e-10 * t) {
      *T = t;
      return it;
    }
  }
  *T = t;
  return -1;
}

}  // namespace orc
