// C ABI of the CPU oracle for the Python test harness (ctypes). TEST INFRASTRUCTURE ONLY.
//
// orc_react_cells restates the per-cell work of the reactor call made at
// Source/PeleLM.cpp:5752 (CGS units, component-major arrays as in
// Source/PeleLM_K.H:11-52): integrate d(rhoY)/dt = W wdot + F_rhoY and the energy equation
// over dt with rho h(t) = rho h0 + F_h t, then recover T from (rho h, Y) and write the RHS
// evaluation count into FC. Cells with mask < 0 are left untouched (FC = 0).
#include <cmath>
#include <cstring>
#include <string>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "chem_oracle.hpp"

using orc::Mechanism;

extern "C" {

void* orc_mech_load(const char* path) {
  auto* m = new Mechanism();
  std::string err;
  if (!m->load(path, &err)) {
    delete m;
    return nullptr;
  }
  return m;
}

void orc_mech_free(void* h) { delete static_cast<Mechanism*>(h); }
int orc_mech_ns(void* h) { return static_cast<Mechanism*>(h)->ns; }
int orc_mech_nr(void* h) { return static_cast<Mechanism*>(h)->nr; }

int orc_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// wdot[c*ns+k] from T[c], C[c*ns+k] (cell-major)
void orc_wdot_cells(void* h, int ncell, const double* T, const double* C, double* wdot) {
  const Mechanism& m = *static_cast<Mechanism*>(h);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncell; ++c) orc::production_rates(m, T[c], C + (size_t)c * m.ns, wdot + (size_t)c * m.ns);
}

// ydot[c*N+i] from y[c*N+i], F[c*ns+k], Fh[c]
void orc_rhs_cells(void* h, int ncell, const double* y, const double* F, const double* Fh,
                   double* ydot) {
  const Mechanism& m = *static_cast<Mechanism*>(h);
  const int N = m.ns + 1;
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncell; ++c)
    orc::reactor_rhs(m, y + (size_t)c * N, F + (size_t)c * m.ns, Fh[c], ydot + (size_t)c * N);
}

void orc_jac(void* h, const double* y, const double* F, double Fh, double* J) {
  orc::reactor_jac(*static_cast<Mechanism*>(h), y, F, Fh, J);
}

void orc_count_rhs(void* h, const double* y, const double* F, double Fh, long* ops, long* trans) {
  orc::count_rhs_ops(*static_cast<Mechanism*>(h), y, F, Fh, ops, trans);
}

double orc_mixture_h(void* h, double T, const double* Y) {
  return orc::mixture_h(*static_cast<Mechanism*>(h), T, Y);
}

// T[c] in/out from h[c] (erg/g) and Y[c*ns+k]
void orc_hy2t_cells(void* h, int ncell, const double* hm, const double* Y, double* T) {
  const Mechanism& m = *static_cast<Mechanism*>(h);
#pragma omp parallel for schedule(static)
  for (int c = 0; c < ncell; ++c) orc::hy2t(m, hm[c], Y + (size_t)c * m.ns, T + c);
}

// Reactor advance of ncell cells, arrays component-major: rY[k*ncell + c].
// stats (optional, per cell, 6 longs): nst nfe nje nlu netf ncfn. Returns #failed cells.
int orc_react_cells(void* h, int ncell, double* rY, const double* rYsrc, double* T, double* rE,
                    const double* rEsrc, double* FC, const int* mask, double dt, double rtol,
                    const double* atol, int max_order, int max_steps, int nthreads, long* stats) {
  const Mechanism& m = *static_cast<Mechanism*>(h);
  const int ns = m.ns, N = ns + 1;
  orc::BdfOptions opt;
  opt.rtol = rtol;
  opt.atol.assign(atol, atol + N);
  opt.max_order = max_order;
  opt.max_steps = max_steps;
  int nfail = 0;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
#pragma omp parallel for schedule(dynamic, 8) reduction(+ : nfail)
  for (int c = 0; c < ncell; ++c) {
    if (mask && mask[c] < 0) {
      FC[c] = 0.0;
      continue;
    }
    double y[orc::MAXNS + 1], F[orc::MAXNS], Y[orc::MAXNS];
    for (int k = 0; k < ns; ++k) {
      y[k] = rY[(size_t)k * ncell + c];
      F[k] = rYsrc[(size_t)k * ncell + c];
    }
    y[ns] = T[c];
    const double Fh = rEsrc[c];
    orc::BdfStats st = orc::bdf_integrate(m, y, F, Fh, dt, opt);
    double rho = 0.0;
    for (int k = 0; k < ns; ++k) {
      rY[(size_t)k * ncell + c] = y[k];
      rho += y[k];
    }
    rE[c] += dt * Fh;
    for (int k = 0; k < ns; ++k) Y[k] = y[k] / rho;
    double Tn = y[ns];
    orc::hy2t(m, rE[c] / rho, Y, &Tn);
    T[c] = Tn;
    FC[c] = (st.status == 0) ? (double)st.nfe : -(double)st.status;
    if (st.status != 0) ++nfail;
    if (stats) {
      long* s = stats + (size_t)c * 6;
      s[0] = st.nst; s[1] = st.nfe; s[2] = st.nje; s[3] = st.nlu; s[4] = st.netf; s[5] = st.ncfn;
    }
  }
  return nfail;
}

// Plain integration of one state vector (for closed-form and scipy cross-checks).
int orc_bdf_one(void* h, double* y, const double* F, double Fh, double dt, double rtol,
                const double* atol, int max_order, int max_steps, long* stats) {
  const Mechanism& m = *static_cast<Mechanism*>(h);
  orc::BdfOptions opt;
  opt.rtol = rtol;
  opt.atol.assign(atol, atol + m.ns + 1);
  opt.max_order = max_order;
  opt.max_steps = max_steps;
  orc::BdfStats st = orc::bdf_integrate(m, y, F, Fh, dt, opt);
  if (stats) {
    stats[0] = st.nst; stats[1] = st.nfe; stats[2] = st.nje; stats[3] = st.nlu;
    stats[4] = st.netf; stats[5] = st.ncfn;
  }
  return st.status;
}

// Dense partial-pivot LU solve of one system with the integrator's factorisation; 0 ok,
// 1 singular.
int orc_lu_solve(int n, const double* A, const double* b, double* x) {
  return orc::lu_solve(n, A, b, x) ? 0 : 1;
}

}  // extern "C"
