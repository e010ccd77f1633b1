// CPU oracle: CVODE-class variable-order, variable-step BDF in Nordsieck form with the
// fixed-leading-coefficient formulation, modified Newton on (I - gamma J) with an analytic
// Jacobian and dense partial-pivot LU, WRMS local error test and step/order selection.
// TEST INFRASTRUCTURE ONLY (see chem_oracle.hpp for scope and parity status).
//
// The method is the published CVODE algorithm (Hindmarsh et al., "SUNDIALS", ACM TOMS
// 31(3) 2005, sec. 2.1; the fixed-leading-coefficient BDF of Jackson & Sacks-Davis, ACM
// TOMS 6(3) 1980; Nordsieck history as in Byrne & Hindmarsh, ACM TOMS 1(1) 1975). The
// reference configures it through cvode.solve_type=denseAJ_direct, cvode.max_order,
// ode.rtol/ode.atol (Exec/RegTests/FlameSheet/inputs.2d-regt:86-91).
//
// Nordsieck array z[j] = h^j y^(j) / j!, j = 0..q. Step n has size h from t_{n-1};
// tau[1] is the last accepted step, tau[2] the one before, etc.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "chem_oracle.hpp"

namespace orc {
namespace {

constexpr int QMAX_ABS = 5;
constexpr double UROUND = DBL_EPSILON;
// step-size / order heuristics (CVODE's documented defaults)
constexpr double ETAMX1 = 10000.0, ETAMX2 = 10.0, ETAMX3 = 10.0, ETAMXF = 0.2;
constexpr double ETAMIN = 0.1, ETACF = 0.25, ADDON = 1e-6;
constexpr double BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, THRESH = 1.5;
constexpr int SMALL_NST = 10, MXNEF = 7, MXNEF1 = 3, SMALL_NEF = 2, MXNCF = 10;
constexpr int MAXCOR = 3, MSBP = 20;
constexpr double CRDOWN = 0.3, RDIV = 2.0, DGMAX = 0.3, NLSCOEF = 0.1;

struct Lu {
  int n = 0;
  std::vector<double> a;
  std::vector<int> piv;
  bool factor() {
    for (int k = 0; k < n; ++k) {
      int p = k;
      double amax = std::fabs(a[k * n + k]);
      for (int i = k + 1; i < n; ++i)
        if (std::fabs(a[i * n + k]) > amax) { amax = std::fabs(a[i * n + k]); p = i; }
      piv[k] = p;
      if (amax == 0.0) return false;
      // swap the trailing part only (multipliers stay in place), so that solve() can apply
      // each interchange just before eliminating its column
      if (p != k)
        for (int j = k; j < n; ++j) std::swap(a[k * n + j], a[p * n + j]);
      const double inv = 1.0 / a[k * n + k];
      for (int i = k + 1; i < n; ++i) {
        const double l = a[i * n + k] * inv;
        a[i * n + k] = l;
        for (int j = k + 1; j < n; ++j) a[i * n + j] -= l * a[k * n + j];
      }
    }
    return true;
  }
  void solve(double* b) const {
    for (int k = 0; k < n; ++k) {
      if (piv[k] != k) std::swap(b[k], b[piv[k]]);
      for (int i = k + 1; i < n; ++i) b[i] -= a[i * n + k] * b[k];
    }
    for (int k = n - 1; k >= 0; --k) {
      for (int j = k + 1; j < n; ++j) b[k] -= a[k * n + j] * b[j];
      b[k] /= a[k * n + k];
    }
  }
};

struct Bdf {
  const Mechanism& m;
  const double* F;
  double Fh;
  const BdfOptions& o;
  int N;
  BdfStats st;
  // Nordsieck history z[0..qmax] plus the saved correction for the order-increase test
  std::vector<double> z[QMAX_ABS + 1], acor_saved, acor, y, ewt, f, tmp, Jm;
  double l[QMAX_ABS + 1] = {0}, tq[6] = {0}, tau[QMAX_ABS + 2] = {0};
  int q = 1, qmax = 5, qwait = 2, qprime = 1;
  double t = 0, h = 0, hscale = 0, eta = 1, etamax = ETAMX1, tq5_saved = 1;
  double gamma = 0, gammap = 0, gamrat = 1, crate = 1, rl1 = 1, acnrm = 0;
  long nstlp = 0;
  int nef = 0, ncf = 0;
  bool force_setup = true;
  Lu lu;

  Bdf(const Mechanism& m_, const double* F_, double Fh_, const BdfOptions& o_)
      : m(m_), F(F_), Fh(Fh_), o(o_), N(m_.ns + 1) {
    qmax = std::max(1, std::min(o.max_order, QMAX_ABS));
    for (auto& v : z) v.assign(N, 0.0);
    acor_saved.assign(N, 0.0); acor.assign(N, 0.0); y.assign(N, 0.0);
    ewt.assign(N, 0.0); f.assign(N, 0.0); tmp.assign(N, 0.0); Jm.assign(N * N, 0.0);
    lu.n = N; lu.a.assign(N * N, 0.0); lu.piv.assign(N, 0);
  }

  void rhs(const double* yy, double* out) { reactor_rhs(m, yy, F, Fh, out); ++st.nfe; }
  void set_ewt(const double* yy) {
    for (int i = 0; i < N; ++i) ewt[i] = 1.0 / (o.rtol * std::fabs(yy[i]) + o.atol[i]);
  }
  double wrms(const double* v) const {
    double s = 0.0;
    for (int i = 0; i < N; ++i) { const double x = v[i] * ewt[i]; s += x * x; }
    return std::sqrt(s / N);
  }
  void rescale(double e) {  // z[j] *= e^j, h *= e
    double fac = e;
    for (int j = 1; j <= q; ++j) {
      for (int i = 0; i < N; ++i) z[j][i] *= fac;
      fac *= e;
    }
    h = hscale * e;
    hscale = h;
  }
  void predict() {
    t += h;
    for (int k = 1; k <= q; ++k)
      for (int j = q; j >= k; --j)
        for (int i = 0; i < N; ++i) z[j - 1][i] += z[j][i];
  }
  void retract() {
    t -= h;
    for (int k = 1; k <= q; ++k)
      for (int j = q; j >= k; --j)
        for (int i = 0; i < N; ++i) z[j - 1][i] -= z[j][i];
  }

  // Coefficients of Lambda(x) (l[]) and the error constants tq[1..5] for order q and
  // step h given the history tau[] (fixed-leading-coefficient BDF).
  void set_coeffs() {
    for (int i = 0; i <= qmax; ++i) l[i] = 0.0;
    l[0] = 1.0;
    double alpha0 = 0.0;
    for (int j = 1; j <= q; ++j) alpha0 -= 1.0 / j;
    double hsum = h, sum_xi_inv = 0.0, xi_inv = 1.0;
    for (int i = 1; i <= q - 1; ++i) {
      if (i > 1) hsum += tau[i - 1];
      xi_inv = h / hsum;
      sum_xi_inv += xi_inv;
      for (int k = i; k >= 1; --k) l[k] += l[k - 1] * xi_inv;
    }
    const double xistar_inv = -alpha0 - sum_xi_inv;
    for (int k = q; k >= 1; --k) l[k] += l[k - 1] * xistar_inv;
    if (q > 1) hsum += tau[q - 1];
    const double xiq_inv = h / hsum;  // 1/xi_q
    const double alpha0_hat = -(sum_xi_inv + xiq_inv);
    const double A1 = 1.0 - alpha0_hat + alpha0;
    const double A2 = 1.0 + q * A1;
    tq[2] = std::fabs(A1 / (alpha0 * A2));
    tq[5] = std::fabs(A2 * xistar_inv / (l[q] * xiq_inv));
    if (qwait == 1) {
      if (q > 1) {
        const double C = xistar_inv / l[q];
        const double A3 = alpha0 + 1.0 / q;
        const double A4 = alpha0_hat + xiq_inv;
        tq[1] = std::fabs(C * (1.0 - A4 + A3) / A3);
      } else {
        tq[1] = 1.0;
      }
      const double xiq1_inv = h / (hsum + tau[q]);
      const double A5 = alpha0 - 1.0 / (q + 1);
      const double A6 = alpha0_hat - xiq1_inv;
      const double Cpp = (1.0 - A6 + A5) / A2;
      tq[3] = std::fabs(Cpp / (xiq1_inv * (q + 2) * A5));
    }
    tq[4] = NLSCOEF / tq[2];
  }

  bool setup_matrix() {  // M = I - gamma J at y
    reactor_jac(m, y.data(), F, Fh, Jm.data());
    ++st.nje;
    for (int i = 0; i < N; ++i)
      for (int j = 0; j < N; ++j) lu.a[i * N + j] = (i == j ? 1.0 : 0.0) - gamma * Jm[i * N + j];
    ++st.nlu;
    gammap = gamma;
    gamrat = 1.0;
    crate = 1.0;
    nstlp = st.nst;
    return lu.factor();
  }

  // Newton iteration; returns 0 converged, 1 recoverable failure, 2 singular matrix
  int newton(bool& jcur) {
    bool call_setup = force_setup || st.nst == 0 || st.nst >= nstlp + MSBP ||
                      std::fabs(gamrat - 1.0) > DGMAX;
    force_setup = false;
    for (;;) {
      for (int i = 0; i < N; ++i) { y[i] = z[0][i]; acor[i] = 0.0; }
      rhs(y.data(), f.data());
      jcur = false;
      if (call_setup) {
        if (!setup_matrix()) return 2;
        jcur = true;
        call_setup = false;
      }
      double delp = 0.0, del = 0.0;
      int mm = 0;
      bool ok = false;
      for (;;) {
        for (int i = 0; i < N; ++i) tmp[i] = gamma * f[i] - (rl1 * z[1][i] + acor[i]);
        lu.solve(tmp.data());
        if (gamrat != 1.0) {
          const double s = 2.0 / (1.0 + gamrat);
          for (int i = 0; i < N; ++i) tmp[i] *= s;
        }
        del = wrms(tmp.data());
        for (int i = 0; i < N; ++i) { acor[i] += tmp[i]; y[i] = z[0][i] + acor[i]; }
        if (mm > 0) crate = std::max(CRDOWN * crate, del / delp);
        const double dcon = del * std::min(1.0, crate) / tq[4];
        if (dcon <= 1.0) {
          acnrm = (mm == 0) ? del : wrms(acor.data());
          ok = true;
          break;
        }
        ++mm;
        if (mm == MAXCOR || (mm >= 2 && del > RDIV * delp)) break;
        delp = del;
        rhs(y.data(), f.data());
        if (!std::isfinite(f[0])) break;
      }
      if (ok) return 0;
      if (!jcur) {  // stale Jacobian: refresh and retry at the same h
        call_setup = true;
        continue;
      }
      return 1;
    }
  }

  void adjust_order(int dq) {
    // xi_j = (t_n - t_{n-j}) / h, from the accepted-step history tau[1..].
    if (dq > 0) {
      // q -> q+1: the new degree-(q+1) polynomial keeps value and slope at t_n and the
      // values at t_{n-1}..t_{n-q+1} (correction term a x^2 prod_{j<q}(x+xi_j)) and also
      // interpolates y_{n-q}, which fixes a = A1 * acor with
      // A1 = (sum_{j<=q} 1/j - sum_{j<=q} 1/xi_j) / prod_{j<=q} xi_j.
      double w[QMAX_ABS + 2] = {0};
      w[2] = 1.0;
      double alpha0 = 0.0, alpha1 = 0.0, prod = 1.0, hsum = 0.0;
      for (int j = 1; j <= q; ++j) {
        hsum += tau[j];
        const double xi = hsum / hscale;
        prod *= xi;
        alpha0 -= 1.0 / j;
        alpha1 += 1.0 / xi;
        if (j <= q - 1)
          for (int i = j + 2; i >= 2; --i) w[i] = w[i] * xi + w[i - 1];
      }
      const double A1 = (-alpha0 - alpha1) / prod;
      for (int i = 0; i < N; ++i) z[q + 1][i] = A1 * acor_saved[i];
      for (int j = 2; j <= q; ++j)
        for (int i = 0; i < N; ++i) z[j][i] += w[j] * z[q + 1][i];
    } else {
      // q -> q-1: drop the top column, keeping value and slope at t_n and the values at
      // t_{n-1}..t_{n-q+2}: subtract z[q] * x^2 prod_{j<=q-2}(x+xi_j).
      double w[QMAX_ABS + 2] = {0};
      w[2] = 1.0;
      double hsum = 0.0;
      for (int j = 1; j <= q - 2; ++j) {
        hsum += tau[j];
        const double xi = hsum / hscale;
        for (int i = j + 2; i >= 2; --i) w[i] = w[i] * xi + w[i - 1];
      }
      for (int j = 2; j < q; ++j)
        for (int i = 0; i < N; ++i) z[j][i] -= w[j] * z[q][i];
      for (int i = 0; i < N; ++i) z[q][i] = 0.0;
    }
  }

  void run(double* yio, double tout) {
    const int ns = m.ns;
    (void)ns;
    for (int i = 0; i < N; ++i) z[0][i] = yio[i];
    t = 0.0;
    // ---- initial step (difference-quotient estimate of y'', bounded) ----
    rhs(z[0].data(), f.data());
    set_ewt(z[0].data());
    const double tdist = tout - t;
    const double tround = UROUND * std::max(std::fabs(t), std::fabs(tout));
    const double hlb = 100.0 * tround;
    double hub_inv = 0.0;
    for (int i = 0; i < N; ++i) {
      const double d = 0.1 * std::fabs(z[0][i]) + o.atol[i];
      hub_inv = std::max(hub_inv, std::fabs(f[i]) / d);
    }
    double hub = 0.1 * tdist;
    if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
    double hg = std::sqrt(hlb * hub), hnew = hg;
    if (hub > hlb) {
      for (int count = 1; count <= 4; ++count) {
        for (int i = 0; i < N; ++i) y[i] = z[0][i] + hg * f[i];
        rhs(y.data(), tmp.data());
        for (int i = 0; i < N; ++i) tmp[i] = (tmp[i] - f[i]) / hg;
        const double ydd = wrms(tmp.data());
        hnew = (ydd * hub * hub > 2.0) ? std::sqrt(2.0 / ydd) : std::sqrt(hg * hub);
        if (count == 4) break;
        const double hrat = hnew / hg;
        if (hrat > 0.5 && hrat < 2.0) break;
        if (count >= 2 && hrat > 2.0) { hnew = hg; break; }
        hg = hnew;
      }
    }
    h = std::min(std::max(0.5 * hnew, hlb), hub);
    hscale = h;
    for (int i = 0; i < N; ++i) z[1][i] = h * f[i];
    q = 1; qwait = 2; etamax = ETAMX1; tau[1] = h;

    // ---- step loop ----
    for (;;) {
      if (st.nst >= o.max_steps) { st.status = 1; break; }
      // never step past tout
      if ((t + h - tout) * h > 0.0) rescale((tout - t) * (1.0 - 4.0 * UROUND) / h);
      set_ewt(z[0].data());
      nef = 0; ncf = 0;
      double dsm = 0.0;
      bool fail_cell = false;
      for (;;) {  // attempt
        predict();
        set_coeffs();
        rl1 = 1.0 / l[1];
        gamma = h * rl1;
        if (st.nst == 0) gammap = gamma;
        gamrat = (st.nst > 0) ? gamma / gammap : 1.0;
        bool jcur = false;
        const int nflag = newton(jcur);
        if (nflag != 0) {
          retract();
          ++ncf; ++st.ncfn;
          if (nflag == 2 || ncf >= MXNCF || std::fabs(h) <= 100.0 * UROUND * std::fabs(t)) {
            st.status = 3; fail_cell = true; break;
          }
          force_setup = true;
          etamax = 1.0;
          rescale(ETACF);
          continue;
        }
        dsm = acnrm * tq[2];
        if (!(dsm <= 1.0)) {  // error test failed (also catches NaN)
          retract();
          ++nef; ++st.netf;
          if (nef >= MXNEF || !std::isfinite(dsm)) { st.status = std::isfinite(dsm) ? 2 : 5; fail_cell = true; break; }
          etamax = 1.0;
          if (nef <= MXNEF1) {
            double e = 1.0 / (std::pow(BIAS2 * dsm, 1.0 / (q + 1)) + ADDON);
            e = std::max(ETAMIN, e);
            if (nef >= SMALL_NEF) e = std::min(e, ETAMXF);
            rescale(e);
          } else if (q > 1) {
            adjust_order(-1);
            --q;
            qwait = q + 1;
            rescale(ETAMIN);
          } else {
            rescale(ETAMIN);
            rhs(z[0].data(), f.data());
            for (int i = 0; i < N; ++i) z[1][i] = h * f[i];
            qwait = 10;
          }
          if (std::fabs(h) <= 100.0 * UROUND * std::fabs(t)) { st.status = 4; fail_cell = true; break; }
          continue;
        }
        break;  // accepted
      }
      if (fail_cell) break;

      // ---- complete the step ----
      ++st.nst;
      for (int i = q + 1; i >= 2; --i) tau[i] = tau[i - 1];
      tau[1] = h;
      for (int j = 0; j <= q; ++j)
        for (int i = 0; i < N; ++i) z[j][i] += l[j] * acor[i];
      --qwait;
      if (qwait == 1 && q != qmax) {
        for (int i = 0; i < N; ++i) acor_saved[i] = acor[i];
        tq5_saved = tq[5];
      }
      if (std::fabs(t - tout) <= 100.0 * UROUND * (std::fabs(t) + std::fabs(h)) || t >= tout) break;

      // ---- choose next step size and order ----
      const double etaq = 1.0 / (std::pow(BIAS2 * dsm, 1.0 / (q + 1)) + ADDON);
      qprime = q;
      if (etamax == 1.0) {
        qwait = std::max(qwait, 2);
        eta = 1.0;
      } else {
        eta = etaq;
        if (qwait == 0) {
          qwait = 2;
          double etaqm1 = 0.0, etaqp1 = 0.0;
          if (q > 1) {
            const double ddn = wrms(z[q].data()) * tq[1];
            etaqm1 = 1.0 / (std::pow(BIAS1 * ddn, 1.0 / q) + ADDON);
          }
          if (q != qmax) {
            const double cquot = (tq[5] / tq5_saved) * std::pow(h / tau[2], q + 1);
            for (int i = 0; i < N; ++i) tmp[i] = acor[i] - cquot * acor_saved[i];
            const double dup = wrms(tmp.data()) * tq[3];
            etaqp1 = 1.0 / (std::pow(BIAS3 * dup, 1.0 / (q + 2)) + ADDON);
          }
          const double etam = std::max(etaqm1, std::max(etaq, etaqp1));
          if (etam < THRESH) {
            eta = 1.0;
          } else if (etam == etaq) {
            eta = etaq;
          } else if (etam == etaqm1) {
            eta = etaqm1; qprime = q - 1;
          } else {
            eta = etaqp1; qprime = q + 1;
            for (int i = 0; i < N; ++i) acor_saved[i] = acor[i];
          }
        } else if (eta < THRESH) {
          eta = 1.0;
        }
        if (eta >= THRESH || qprime != q) eta = std::min(eta, etamax);
        else eta = 1.0;
      }
      etamax = (st.nst <= SMALL_NST) ? ETAMX2 : ETAMX3;
      if (qprime != q) {
        adjust_order(qprime - q);
        q = qprime;
        qwait = q + 1;
      }
      if (eta != 1.0) rescale(eta);
    }
    for (int i = 0; i < N; ++i) yio[i] = z[0][i];
  }
};

}  // namespace

BdfStats bdf_integrate(const Mechanism& m, double* y, const double* F, double Fh, double dt,
                       const BdfOptions& opt) {
  Bdf b(m, F, Fh, opt);
  b.run(y, dt);
  return b.st;
}

bool lu_solve(int n, const double* A, const double* b, double* x) {
  Lu lu;
  lu.n = n;
  lu.a.assign(A, A + (size_t)n * n);
  lu.piv.assign(n, 0);
  if (!lu.factor()) return false;
  for (int i = 0; i < n; ++i) x[i] = b[i];
  lu.solve(x);
  return true;
}

}  // namespace orc
