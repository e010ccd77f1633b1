// CPU oracle: table-driven restatement of the chemistry path. TEST INFRASTRUCTURE ONLY —
// used by tests/, the smoke check and the CPU baseline leg of bench.py, never by the
// product library.
//
// Parity status: the reference's own implementation of this path (PelePhysics reactors,
// FUEGO mechanisms, SUNDIALS CVODE) is absent from the reference tree (empty submodules),
// and the reference ships no golden vectors for the reactor. Parity is therefore
// UNPINNED against the reference; the oracle is pinned against closed-form known-answer
// tests and cross-checked against scipy's VODE BDF (see tests/golden).
//
// Follows:
//   kinetics + thermo equations      Docs/source/manual/Model.rst:227-296
//   reaction ODE with frozen sources Docs/source/manual/Model.rst:675-691
//   per-cell packing / CGS units     Source/PeleLM_K.H:11-52, Source/PeleLM.cpp:5736-5771
//   T from (h, Y) Newton             Source/PeleLM_K.H:508-529, Source/PeleLM.cpp:8201-8287
//   BDF integrator                   published CVODE algorithm (Hindmarsh et al., ACM TOMS
//                                    31(3) 2005; Jackson & Sacks-Davis, ACM TOMS 6(3) 1980;
//                                    Byrne & Hindmarsh, ACM TOMS 1(1) 1975)
#pragma once
#include <array>
#include <cmath>
#include <string>
#include <utility>
#include <vector>

namespace orc {

constexpr double R_ERG = 8.31446261815324e7;   // erg/mol/K
constexpr double R_CAL = 1.98720425864083;     // cal/mol/K
constexpr double P_ATM = 1.01325e6;            // dyn/cm^2
constexpr int MAXNS = 64;
constexpr int MAXNR = 400;

struct Reaction {
  int kind = 0;  // 0 elementary, 1 three-body, 2 falloff
  bool reversible = true;
  std::vector<std::pair<int, int>> reac, prod;
  double A = 0, beta = 0, Ea = 0;     // k (or k_inf)
  double A0 = 0, beta0 = 0, Ea0 = 0;  // k_0 (falloff)
  std::vector<double> troe;           // empty => Lindemann
  std::vector<std::pair<int, double>> eff;  // third-body efficiencies (default 1)
  double lnA = 0, lnA0 = 0;           // derived at load
  int dnu = 0;                        // sum(nu'') - sum(nu')
};

struct Mechanism {
  int ns = 0, nr = 0, nel = 0;
  std::vector<double> W, Tmid;
  std::vector<std::array<double, 7>> lo, hi;
  std::vector<std::vector<std::pair<int, int>>> comp;
  std::vector<Reaction> rx;
  bool load(const std::string& path, std::string* err);
};

// Thermo for one species at T (per mole, dimensionless).
void species_thermo(const Mechanism& m, int k, double T, double* cpR, double* hRT, double* sR,
                    double* dcpRdT);

// Molar production rates wdot [mol/cm^3/s] from T and concentrations C [mol/cm^3].
void production_rates(const Mechanism& m, double T, const double* C, double* wdot);

// Reactor RHS: y = [rhoY_k (g/cm^3), T], F = forcing on rhoY (g/cm^3/s), Fh forcing on rho h.
void reactor_rhs(const Mechanism& m, const double* y, const double* F, double Fh, double* ydot);

// Algorithmic op count of one reactor_rhs evaluation (add/sub/mul/div; transcendentals
// exp/log/log10/pow counted separately).
void count_rhs_ops(const Mechanism& m, const double* y, const double* F, double Fh, long* ops,
                   long* trans);

// Analytic Jacobian d ydot / d y, row-major N x N (N = ns+1).
void reactor_jac(const Mechanism& m, const double* y, const double* F, double Fh, double* J);

// Mass-specific enthalpy of the mixture [erg/g] at T for mass fractions Y.
double mixture_h(const Mechanism& m, double T, const double* Y);
// T from (h [erg/g], Y) by Newton; returns iterations (<0 on failure).
int hy2t(const Mechanism& m, double h, const double* Y, double* T);

struct BdfOptions {
  double rtol = 1e-6;
  std::vector<double> atol;  // size N
  int max_order = 5;
  int max_steps = 20000;
};

struct BdfStats {
  long nst = 0, nfe = 0, nje = 0, nlu = 0, netf = 0, ncfn = 0;
  int status = 0;  // 0 ok, 1 max steps, 2 error-test failures, 3 convergence failures, 4 h too small, 5 nonfinite
};

// Integrate one cell over [0, dt] (constant-pressure RhoH reactor). y in/out.
BdfStats bdf_integrate(const Mechanism& m, double* y, const double* F, double Fh, double dt,
                       const BdfOptions& opt);

// The integrator's dense partial-pivot LU applied to one system A x = b (A row-major n x n);
// false when a pivot column is zero (singular). For the LU known-answer tests.
bool lu_solve(int n, const double* A, const double* b, double* x);

}  // namespace orc
