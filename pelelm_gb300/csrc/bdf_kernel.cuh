// Persistent, work-stealing, cell-per-thread BDF reactor kernel.
//
// Replaces the per-cell integration inside the PelePhysics reactor called at
// Source/PeleLM.cpp:5752 (CVODE BDF with an analytic Jacobian and dense direct solve,
// cvode.solve_type = denseAJ_direct, Exec/RegTests/FlameSheet/inputs.2d-regt:86-91).
// The algorithm is the CVODE-class fixed-leading-coefficient BDF in Nordsieck form
// (Hindmarsh et al., ACM TOMS 31(3) 2005; Jackson & Sacks-Davis, ACM TOMS 6(3) 1980);
// its CPU statement is oracle/bdf_oracle.cpp and this kernel makes the same decisions.
//
// GB300 mapping:
//  * FP64 issue is ~1/74 of FP32 on this part and an FP64 warp instruction costs the same
//    whatever its active mask, so the kernel is a flattened per-thread state machine in
//    which every pass runs exactly one FP64 right-hand side for all lanes (convergent);
//    step start / Newton update / step completion are short predicated tails.
//  * The Jacobian and its LU (type JR) run in FP32 in mixed mode (inexact Newton; residual,
//    error test and step control stay FP64) or FP64 in plain mode.
//  * Lanes whose cell is finished take the next cell from a global queue with one
//    warp-aggregated atomic (work stealing across all boxes of all levels), so stiff cells
//    with hundreds of substeps never hold back quiescent ones.
//  * Nordsieck history, forcing and the LU live in shared memory laid out
//    [element][thread] (each warp access is contiguous, bank-conflict free); the state,
//    correction and error weights live in registers (N is a compile-time constant).
//  * With a retry list (mixed precision), a cell whose integration fails is listed and its
//    arrays are left as they were, for the FP64 pass that follows on the same stream.
#ifndef PGB_BDF_KERNEL_CUH
#define PGB_BDF_KERNEL_CUH

#include <float.h>

#include "mech_common.cuh"
#include "mech_tables.cuh"
#include "reactor_types.cuh"

namespace pgb {

namespace bdf {
constexpr double UROUND = DBL_EPSILON;
constexpr double ETAMX1 = 10000.0, ETAMX2 = 10.0, ETAMX3 = 10.0, ETAMXF = 0.2;
constexpr double ETAMIN = 0.1, ETACF = 0.25, ADDON = 1e-6;
constexpr double BIAS1 = 6.0, BIAS2 = 6.0, BIAS3 = 10.0, THRESH = 1.5;
constexpr int SMALL_NST = 10, MXNEF = 7, MXNEF1 = 3, SMALL_NEF = 2, MXNCF = 10;
constexpr int MAXCOR = 3, MSBP = 20;
constexpr double CRDOWN = 0.3, RDIV = 2.0, DGMAX = 0.3, NLSCOEF = 0.1;

// FINISH: the cell's integration has ended (status set) and its write-back is pending; the
// group kernel runs that write-back from one place at the end of a pass (the per-thread kernel,
// whose cells finish where they end, does not use it).
enum Phase : int { IDLE = 0, NEED = 1, FINISH = 2, START = 3, HIN = 4, STEP = 5, NEWTON = 6, RESETD = 7 };

// 1/j for the small integers the order logic divides by (no FP64 division on the device)
__device__ __forceinline__ double inv_int(int j) {
  return j == 1 ? 1.0 : j == 2 ? 0.5 : j == 3 ? 1.0 / 3.0 : j == 4 ? 0.25 : j == 5 ? 0.2
       : j == 6 ? 1.0 / 6.0 : 1.0 / 7.0;
}

// 1/x to ~1e-14 from an FP32 seed and one Newton step (3 FP64-pipe instructions instead of a
// 7-8 slot IEEE division); used for error weights in mixed precision. x must lie in the
// normal FP32 range.
__device__ __forceinline__ double recip_fast(double x) {
  const double y0 = (double)__frcp_rn((float)x);
  return fma(y0, fma(-x, y0, 1.0), y0);
}
enum Status : int { OK = 0, MAX_STEPS = 1, ERRTEST = 2, CONV = 3, HSMALL = 4, NONFINITE = 5 };
}  // namespace bdf

// Where the per-thread arrays live: shared memory by default; LAYOUT_LU_GLOBAL puts the
// Jacobian/LU slice and LAYOUT_Z_GLOBAL the Nordsieck history into L2-resident global scratch
// (ReactParams::lu_scratch / z_scratch, each an [element][slot] array over all resident
// threads, so a warp's access to one element is one contiguous 256 B line).
enum : int { LAYOUT_LU_GLOBAL = 1, LAYOUT_Z_GLOBAL = 2 };

// Bytes of dynamic shared memory per thread for mechanism M, Jacobian type JR and LAYOUT.
template <class M, class JR, int LAYOUT = 0>
__host__ __device__ constexpr int bdf_smem_per_thread() {
  return ((LAYOUT & LAYOUT_Z_GLOBAL) ? 0 : (QMAX + 2) * M::N * 8)  // Nordsieck + saved correction
         + (QMAX + 1) * 8         // l coefficients
         + (QMAX + 2) * 8         // step history tau
         + M::N * 8               // forcing (F_rhoY, F_rhoh)
         + M::N * (int)sizeof(JR)  // triangular-solve vector
         + ((LAYOUT & LAYOUT_LU_GLOBAL) ? 0 : M::N * M::N * (int)sizeof(JR))  // Jacobian / LU
         + (M::RHS_TABLE ? 3 * M::NS * 8 : 0)  // table RHS: concentrations, g/RT, production
         + ((M::N + 7) / 8) * 8;  // pivots
}

template <class JR>
struct LuAcc {  // J(i,k) view of one thread's matrix slice, element stride `stride`
  JR* base;
  int n;
  long long stride;
  __device__ __forceinline__ JR& operator()(int i, int k) const {
    return base[(long long)(i * n + k) * stride];
  }
};

template <class M, class JR, int TPB, int LAYOUT = 0>
__global__ void __launch_bounds__(TPB, 1) bdf_reactor_kernel(const ReactParams P) {
  constexpr bool LU_GLOBAL = (LAYOUT & LAYOUT_LU_GLOBAL) != 0;
  constexpr bool Z_GLOBAL = (LAYOUT & LAYOUT_Z_GLOBAL) != 0;
  using namespace bdf;
  constexpr bool MIXED = sizeof(JR) == sizeof(float);
  constexpr int N = M::N;
  constexpr int NS = M::NS;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  const int tid = threadIdx.x;
  const int lane = tid & 31;
  double* const smem_d = reinterpret_cast<double*>(smem_raw);
  double* Zs = smem_d;                                           // [(QMAX+2)*N][TPB] unless global
  double* Ls = Z_GLOBAL ? smem_d : Zs + (QMAX + 2) * N * TPB;    // [QMAX+1][TPB]
  double* TAUs = Ls + (QMAX + 1) * TPB;                          // [QMAX+2][TPB]
  double* Fs = TAUs + (QMAX + 2) * TPB;                          // [N][TPB]
  JR* XSs = reinterpret_cast<JR*>(Fs + N * TPB);                 // [N][TPB] solve vector
  JR* LUs = XSs + N * TPB;                                       // [N*N][TPB] unless global
  double* RSs = reinterpret_cast<double*>(LU_GLOBAL ? LUs : LUs + N * N * TPB);  // [3*NS][TPB] table RHS
  unsigned char* PIVs = reinterpret_cast<unsigned char*>(RSs + (M::RHS_TABLE ? 3 * NS * TPB : 0));
  const long long slot = (long long)blockIdx.x * TPB + tid;
  const long long nslot = (long long)gridDim.x * TPB;
  // this thread's Jacobian / LU slice and Nordsieck slice, with their element strides
  JR* const LUb = LU_GLOBAL ? static_cast<JR*>(P.lu_scratch) + slot : LUs + tid;
  const long long lu_stride = LU_GLOBAL ? nslot : (long long)TPB;
  double* const Zb = Z_GLOBAL ? static_cast<double*>(P.z_scratch) + slot : Zs + tid;
  const long long z_stride = Z_GLOBAL ? nslot : (long long)TPB;
#define Z(j, i) Zb[(long long)((j) * N + (i)) * z_stride]
#define LCO(j) Ls[(j) * TPB + tid]
#define TAU(j) TAUs[(j) * TPB + tid]
#define FRC(i) Fs[(i) * TPB + tid]
#define LU(i, k) LUb[(long long)((i) * N + (k)) * lu_stride]
#define PIV(k) PIVs[(k) * TPB + tid]
#define XS(i) XSs[(i) * TPB + tid]
  const int qmax = max(1, min(P.max_order, QMAX));
  const double tout = P.dt;

  // ---- per-lane state ----
  int phase = NEED;
  long long cell = -1;
  const long long ncell = P.ncell_dev ? (long long)*P.ncell_dev : P.ncell;
  int box = 0, ci = 0, cj = 0, ck = 0;
  double y[N], acor[N], ewt[N];
  double t = 0.0, h = 0.0, hscale = 0.0, etamax = ETAMX1, eta = 1.0;
  double gamma = 0.0, gammap = 0.0, gamrat = 1.0, crate2 = 1.0, rl1 = 1.0;
  // tq1..tq5: error constants; the Newton test constant tq4 = NLSCOEF/tq2 is kept as 1/tq4^2
  double tq1 = 1.0, tq2 = 1.0, tq3 = 1.0, tq5 = 1.0, tq5_saved = 1.0, inv_tq4_sq = 1.0;
  // del2/delp2: squared WRMS norms of the last / previous Newton corrections; crate2 = crate^2
  double del2 = 0.0, delp2 = 0.0, hg = 0.0, hub = 0.0, hlb = 0.0, rE0 = 0.0;
  int q = 1, qwait = 2, nef = 0, ncf = 0, m = 0, hin_count = 0, status = OK;
  long long nst = 0, nfe = 0, nje = 0, nstlp = 0, netf = 0, ncfn = 0;
  bool new_step = true, need_setup = true, force_setup = true, jcur = false;

#pragma unroll
  for (int i = 0; i < N; ++i) { y[i] = 0.0; acor[i] = 0.0; ewt[i] = 1.0; }

  // weighted mean square (the square of CVODE's WRMS norm): every test below compares squares,
  // so no FP64 square root is taken on the step path
  auto wms = [&](const double* v) -> double {
    double s = 0.0;
#pragma unroll
    for (int i = 0; i < N; ++i) { const double x = v[i] * ewt[i]; s = fma(x, x, s); }
    return s * (1.0 / N);
  };
  auto set_ewt = [&]() {
#pragma unroll
    for (int i = 0; i < N; ++i) {
      const double d = fma(P.rtol, fabs(Z(0, i)), P.atol[i]);
      ewt[i] = MIXED ? recip_fast(d) : 1.0 / d;
    }
  };
  auto rescale = [&](double e) {
    double fac = e;
    for (int j = 1; j <= q; ++j) {
#pragma unroll
      for (int i = 0; i < N; ++i) Z(j, i) *= fac;
      fac *= e;
    }
    h = hscale * e;
    hscale = h;
  };
  auto predict = [&]() {
    t += h;
    for (int k = 1; k <= q; ++k)
      for (int j = q; j >= k; --j) {
#pragma unroll
        for (int i = 0; i < N; ++i) Z(j - 1, i) += Z(j, i);
      }
  };
  auto retract = [&]() {
    t -= h;
    for (int k = 1; k <= q; ++k)
      for (int j = q; j >= k; --j) {
#pragma unroll
        for (int i = 0; i < N; ++i) Z(j - 1, i) -= Z(j, i);
      }
  };
  // fixed-leading-coefficient BDF: Lambda(x) coefficients l[] and error constants tq1..tq5
  auto set_coeffs = [&]() {
    for (int i = 0; i <= qmax; ++i) LCO(i) = 0.0;
    LCO(0) = 1.0;
    double alpha0 = 0.0;
    for (int j = 1; j <= q; ++j) alpha0 -= inv_int(j);
    double hsum = h, sum_xi_inv = 0.0;
    for (int i = 1; i <= q - 1; ++i) {
      if (i > 1) hsum += TAU(i - 1);
      const double xi_inv = h / hsum;
      sum_xi_inv += xi_inv;
      for (int k = i; k >= 1; --k) LCO(k) += LCO(k - 1) * xi_inv;
    }
    const double xistar_inv = -alpha0 - sum_xi_inv;
    for (int k = q; k >= 1; --k) LCO(k) += LCO(k - 1) * xistar_inv;
    if (q > 1) hsum += TAU(q - 1);
    const double xiq_inv = h / hsum;
    const double alpha0_hat = -(sum_xi_inv + xiq_inv);
    const double A1 = 1.0 - alpha0_hat + alpha0;
    const double A2 = 1.0 + q * A1;
    tq2 = fabs(A1 / (alpha0 * A2));
    tq5 = fabs(A2 * xistar_inv / (LCO(q) * xiq_inv));
    if (qwait == 1) {
      if (q > 1) {
        const double C = xistar_inv / LCO(q);
        const double A3 = alpha0 + inv_int(q);
        const double A4 = alpha0_hat + xiq_inv;
        tq1 = fabs(C * (1.0 - A4 + A3) / A3);
      } else {
        tq1 = 1.0;
      }
      const double xiq1_inv = h / (hsum + TAU(q));
      const double A5 = alpha0 - inv_int(q + 1);
      const double A6 = alpha0_hat - xiq1_inv;
      const double Cpp = (1.0 - A6 + A5) / A2;
      tq3 = fabs(Cpp / (xiq1_inv * (q + 2) * A5));
    }
    inv_tq4_sq = (tq2 * (1.0 / NLSCOEF)) * (tq2 * (1.0 / NLSCOEF));
  };
  auto adjust_order = [&](int dq) {
    double w[QMAX + 2];
    for (int i = 0; i < QMAX + 2; ++i) w[i] = 0.0;
    w[2] = 1.0;
    if (dq > 0) {
      double alpha0 = 0.0, alpha1 = 0.0, prod = 1.0, hsum = 0.0;
      for (int j = 1; j <= q; ++j) {
        hsum += TAU(j);
        const double xi = hsum / hscale;
        prod *= xi;
        alpha0 -= inv_int(j);
        alpha1 += 1.0 / xi;
        if (j <= q - 1)
          for (int i = j + 2; i >= 2; --i) w[i] = w[i] * xi + w[i - 1];
      }
      const double A1 = (-alpha0 - alpha1) / prod;
#pragma unroll
      for (int i = 0; i < N; ++i) Z(q + 1, i) = A1 * Z(QMAX + 1, i);
      for (int j = 2; j <= q; ++j) {
        const double wj = w[j];
#pragma unroll
        for (int i = 0; i < N; ++i) Z(j, i) = fma(wj, Z(q + 1, i), Z(j, i));
      }
    } else {
      double hsum = 0.0;
      for (int j = 1; j <= q - 2; ++j) {
        hsum += TAU(j);
        const double xi = hsum / hscale;
        for (int i = j + 2; i >= 2; --i) w[i] = w[i] * xi + w[i - 1];
      }
      for (int j = 2; j < q; ++j) {
        const double wj = w[j];
#pragma unroll
        for (int i = 0; i < N; ++i) Z(j, i) = fma(-wj, Z(q, i), Z(j, i));
      }
#pragma unroll
      for (int i = 0; i < N; ++i) Z(q, i) = 0.0;
    }
  };
  // M = I - gamma J in the LU slice, factor with partial pivoting (trailing swaps)
  auto setup_matrix = [&]() -> bool {
    LuAcc<JR> acc{LUb, N, lu_stride};
    if constexpr (M::JAC_TABLE) {
      // concentrations go to the solve vector (free during the setup); forcing read in place
      jac_table<typename M::Tab, JR>(y, [&](int k) -> double { return FRC(k); }, FRC(NS), acc,
                                     [&](int k) -> JR& { return XS(k); });
    } else {
      double Fl[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) Fl[i] = FRC(i);
      M::template jac<JR>(y, Fl, FRC(NS), acc);
    }
    const JR g = (JR)gamma;
#pragma unroll 1
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < N; ++k) LU(i, k) = (i == k ? JR(1) : JR(0)) - g * LU(i, k);
    bool ok = true;
    // partial-pivot LU; the diagonal keeps the reciprocal pivot for the solve
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
      int p = k;
      JR amax = fabs(LU(k, k));
      for (int i = k + 1; i < N; ++i) {
        const JR v = fabs(LU(i, k));
        if (v > amax) { amax = v; p = i; }
      }
      PIV(k) = (unsigned char)p;
      if (!(amax > JR(0))) { ok = false; break; }
      if (p != k)
        for (int j = k; j < N; ++j) { const JR tmp = LU(k, j); LU(k, j) = LU(p, j); LU(p, j) = tmp; }
      const JR inv = JR(1) / LU(k, k);
      LU(k, k) = inv;
      for (int i = k + 1; i < N; ++i) {
        const JR l = LU(i, k) * inv;
        LU(i, k) = l;
        for (int j = k + 1; j < N; ++j) LU(i, j) -= l * LU(k, j);
      }
    }
    ++nje;
    gammap = gamma;
    gamrat = 1.0;
    crate2 = 1.0;
    nstlp = nst;
    return ok;
  };
  // (I - gamma J) x = b with the factors above; the vector lives in shared memory so the
  // row interchanges are plain indexed accesses
  auto lu_solve = [&](double* b) {
#pragma unroll
    for (int i = 0; i < N; ++i) XS(i) = (JR)b[i];
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
      const int p = PIV(k);
      if (p != k) { const JR tmp = XS(k); XS(k) = XS(p); XS(p) = tmp; }
      const JR bk = XS(k);
      for (int i = k + 1; i < N; ++i) XS(i) -= LU(i, k) * bk;
    }
#pragma unroll 1
    for (int k = N - 1; k >= 0; --k) {
      JR sacc = XS(k);
      for (int j = k + 1; j < N; ++j) sacc -= LU(k, j) * XS(j);
      XS(k) = sacc * LU(k, k);
    }
#pragma unroll
    for (int i = 0; i < N; ++i) b[i] = (double)XS(i);
  };
  // ---- cell I/O ----
  auto elem = [&](const ArrDev& a, int n) -> double& {
    return a.p[(long long)(ci - a.begin0) + (long long)(cj - a.begin1) * a.jstride +
               (long long)(ck - a.begin2) * a.kstride + (long long)n * a.nstride];
  };
  auto finish_cell = [&]() {
    const BoxDev& B = P.boxes[box];
    if (status != OK && P.retry_list) {  // hand the cell to the retry pass, arrays untouched
      P.retry_list[atomicAdd(P.retry_count, 1ull)] = cell;
      ReactStats* S = P.stats;
      atomicAdd(&S->nst, (unsigned long long)nst);
      atomicAdd(&S->nfe, (unsigned long long)nfe);
      atomicAdd(&S->nje, (unsigned long long)nje);
      atomicAdd(&S->netf, (unsigned long long)netf);
      atomicAdd(&S->ncfn, (unsigned long long)ncfn);
      atomicAdd(&S->nretry, 1ull);
      phase = NEED;
      return;
    }
    // rho h(t) = rho h0 + F_h t ; T from (h, Y) by Newton with the integrated T as guess
    const double rE = fma(tout, FRC(NS), rE0);
    double rho = 0.0;
#pragma unroll
    for (int k = 0; k < NS; ++k) rho += Z(0, k);
    const double inv_rho = 1.0 / rho;
    double Yk[NS];
#pragma unroll
    for (int k = 0; k < NS; ++k) Yk[k] = Z(0, k) * inv_rho;
    const double htarget = rE * inv_rho;
    double Tn = Z(0, NS);
    if (!(Tn > 90.0 && Tn < 5000.0)) Tn = 1000.0;
    for (int it = 0; it < 50; ++it) {
      double hh, cp;
      M::h_cp_mix(Tn, Yk, hh, cp);
      double dT = (htarget - hh) / cp;
      dT = fmax(-100.0, fmin(100.0, dT));
      Tn = fmax(90.0, fmin(5000.0, Tn + dT));
      if (fabs(dT) < 1e-10 * Tn) break;
    }
    if (B.IR.p) {
      const double dt_inv = 1.0 / tout;
#pragma unroll
      for (int k = 0; k < NS; ++k)  // separate roundings, as separate passes over arrays give
        elem(B.IR, k) = __dsub_rn(__dmul_rn(-__dsub_rn(elem(B.rY, k), __dmul_rn(Z(0, k), B.sY_out)), dt_inv),
                                  elem(B.rYsrc, k));
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) elem(B.rY, k) = Z(0, k) * B.sY_out;
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
    phase = NEED;
  };
  auto fail_cell = [&](int st) {
    status = st;
    finish_cell();
  };
  auto load_cell = [&](long long c) {
    // box containing flat cell c (binary search over cell offsets)
    int lo = 0, hi = P.nbox - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (P.boxes[mid].cell_offset <= c) lo = mid; else hi = mid - 1;
    }
    box = lo;
    const BoxDev& B = P.boxes[box];
    long long r = c - B.cell_offset;
    const int nx = B.len0, ny = B.len1;
    ci = B.lo0 + (int)(r % nx);
    r /= nx;
    cj = B.lo1 + (int)(r % ny);
    ck = B.lo2 + (int)(r / ny);
    if (B.mask.p) {
      const int mv = B.mask.p[(long long)(ci - B.mask.begin0) + (long long)(cj - B.mask.begin1) * B.mask.jstride +
                              (long long)(ck - B.mask.begin2) * B.mask.kstride];
      if (mv < 0) {  // covered cell: no reaction, zero function count
        elem(B.FC, 0) = 0.0;
        if (B.IR.p)
          for (int k = 0; k < NS; ++k) elem(B.IR, k) = -elem(B.rYsrc, k);
        return false;
      }
    }
#pragma unroll
    for (int k = 0; k < NS; ++k) {
      Z(0, k) = elem(B.rY, k) * B.sY_in;
      FRC(k) = elem(B.rYsrc, k) * B.sY_in;
    }
    Z(0, NS) = elem(B.T, 0);
    FRC(NS) = elem(B.rEsrc, 0) * B.sE_in;
    rE0 = elem(B.rE, 0) * B.sE_in;
    for (int j = 1; j <= QMAX + 1; ++j)
#pragma unroll
      for (int i = 0; i < N; ++i) Z(j, i) = 0.0;
    for (int j = 0; j <= QMAX + 1; ++j) TAU(j) = 0.0;
    t = 0.0; h = 0.0; hscale = 0.0; etamax = ETAMX1; eta = 1.0;
    gamma = 0.0; gammap = 0.0; gamrat = 1.0; crate2 = 1.0; rl1 = 1.0;
    tq1 = tq2 = tq3 = tq5 = tq5_saved = inv_tq4_sq = 1.0;
    q = 1; qwait = 2; nef = 0; ncf = 0; m = 0; status = OK;
    nst = 0; nfe = 0; nje = 0; nstlp = 0; netf = 0; ncfn = 0;
    new_step = true; need_setup = true; force_setup = true; jcur = false;
    return true;
  };

  for (;;) {
    // ------------------------------------------------ (A) work stealing
    const unsigned need = __ballot_sync(0xffffffffu, phase == NEED);
    if (need) {
      const int leader = __ffs(need) - 1;
      unsigned long long base = 0;
      if (lane == leader) base = atomicAdd(P.next_cell, (unsigned long long)__popc(need));
      base = __shfl_sync(0xffffffffu, base, leader);
      if (phase == NEED) {
        const long long c = (long long)base + __popc(need & ((1u << lane) - 1u));
        if (c >= ncell) {
          phase = IDLE;
        } else {
          cell = P.cell_list ? P.cell_list[c] : c;
          if (load_cell(cell)) phase = START;  // masked cells stay NEED and refetch next pass
        }
      }
    }
    if (__all_sync(0xffffffffu, phase == IDLE)) break;

    // ------------------------------------------------ (B) prepare the RHS argument
    if (phase == STEP) {
      bool ok = true;
      if (new_step) {
        if (nst >= P.max_steps) { fail_cell(MAX_STEPS); ok = false; }
        else {
          if ((t + h - tout) * h > 0.0) rescale((tout - t) * (1.0 - 4.0 * UROUND) / h);
          set_ewt();
          nef = 0; ncf = 0;
          new_step = false;
        }
      }
      if (ok) {
        predict();
        set_coeffs();
        rl1 = 1.0 / LCO(1);
        gamma = h * rl1;
        if (nst == 0) gammap = gamma;
        gamrat = (nst > 0) ? gamma / gammap : 1.0;
        need_setup = force_setup || nst == 0 || nst >= nstlp + MSBP || fabs(gamrat - 1.0) > DGMAX;
        force_setup = false;
        jcur = false;
        m = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) { y[i] = Z(0, i); acor[i] = 0.0; }
        phase = NEWTON;
      }
    } else if (phase == HIN) {
#pragma unroll
      for (int i = 0; i < N; ++i) y[i] = fma(hg, Z(1, i), Z(0, i));
    } else if (phase == START || phase == RESETD) {
#pragma unroll
      for (int i = 0; i < N; ++i) y[i] = Z(0, i);
    }

    // ------------------------------------------------ (C) one FP64 RHS for every lane
    double f[N];
    const bool active = phase >= START;
    if (active) {
      if constexpr (M::RHS_TABLE) {
        rhs_table<typename M::Tab>(y, [&](int k) -> double { return FRC(k); }, FRC(NS), f,
                                   [&](int k) -> double& { return RSs[k * TPB + tid]; },
                                   [&](int k) -> double& { return RSs[(NS + k) * TPB + tid]; },
                                   [&](int k) -> double& { return RSs[(2 * NS + k) * TPB + tid]; });
      } else {
        double Fl[NS];
#pragma unroll
        for (int i = 0; i < NS; ++i) Fl[i] = FRC(i);
        M::rhs(y, Fl, FRC(NS), f);
      }
      ++nfe;
    }

    // ------------------------------------------------ (D) consume it
    if (phase == START) {
      // initial step size: difference-quotient estimate of y'' (bounded)
#pragma unroll
      for (int i = 0; i < N; ++i) Z(1, i) = f[i];  // f0 parked in z[1] until h is known
      set_ewt();
      const double tround = UROUND * tout;
      hlb = 100.0 * tround;
      double hub_inv = 0.0;
#pragma unroll
      for (int i = 0; i < N; ++i)
        hub_inv = fmax(hub_inv, fabs(f[i]) / fma(0.1, fabs(Z(0, i)), P.atol[i]));
      hub = 0.1 * tout;
      if (hub * hub_inv > 1.0) hub = 1.0 / hub_inv;
      hg = sqrt(hlb * hub);
      if (hub > hlb) {
        hin_count = 1;
        phase = HIN;
      } else {
        h = fmin(fmax(0.5 * hg, hlb), hub);
        hscale = h;
#pragma unroll
        for (int i = 0; i < N; ++i) Z(1, i) *= h;
        q = 1; qwait = 2; etamax = ETAMX1; TAU(1) = h; new_step = true;
        phase = STEP;
      }
    } else if (phase == HIN) {
      double d[N];
#pragma unroll
      for (int i = 0; i < N; ++i) d[i] = (f[i] - Z(1, i)) / hg;
      const double ydd = sqrt(wms(d));
      double hnew = (ydd * hub * hub > 2.0) ? sqrt(2.0 / ydd) : sqrt(hg * hub);
      bool done = false;
      if (hin_count == 4) {
        done = true;
      } else {
        const double hrat = hnew / hg;
        if (hrat > 0.5 && hrat < 2.0) done = true;
        else if (hin_count >= 2 && hrat > 2.0) { hnew = hg; done = true; }
        else { hg = hnew; ++hin_count; }
      }
      if (done) {
        h = fmin(fmax(0.5 * hnew, hlb), hub);
        hscale = h;
#pragma unroll
        for (int i = 0; i < N; ++i) Z(1, i) *= h;
        q = 1; qwait = 2; etamax = ETAMX1; TAU(1) = h; new_step = true;
        phase = STEP;
      }
    } else if (phase == RESETD) {
#pragma unroll
      for (int i = 0; i < N; ++i) Z(1, i) = h * f[i];
      phase = STEP;
    } else if (phase == NEWTON) {
      bool singular = false;
      if (m == 0 && need_setup) {
        singular = !setup_matrix();
        need_setup = false;
        jcur = true;
      }
      int outcome = 0;  // 0 continue, 1 converged, 2 convergence failure
      if (singular) {
        outcome = 3;
      } else {
        double b[N];
#pragma unroll
        for (int i = 0; i < N; ++i) b[i] = fma(gamma, f[i], -fma(rl1, Z(1, i), acor[i]));
        lu_solve(b);
        if (gamrat != 1.0) {
          const double s = 2.0 / (1.0 + gamrat);
#pragma unroll
          for (int i = 0; i < N; ++i) b[i] *= s;
        }
        del2 = wms(b);
#pragma unroll
        for (int i = 0; i < N; ++i) { acor[i] += b[i]; y[i] = Z(0, i) + acor[i]; }
        if (m > 0) crate2 = fmax((CRDOWN * CRDOWN) * crate2, del2 / delp2);
        // convergence: del * min(1, crate) / tq4 <= 1, in squares
        const double dcon2 = del2 * fmin(1.0, crate2) * inv_tq4_sq;
        if (dcon2 <= 1.0) {
          outcome = 1;
        } else {
          ++m;
          if (m == MAXCOR || (m >= 2 && del2 > (RDIV * RDIV) * delp2)) outcome = 2;
          else delp2 = del2;
        }
      }
      if (outcome == 2 && !jcur) {
        // stale Jacobian: refresh it and restart the iteration from the prediction
        need_setup = true;
        m = 0;
#pragma unroll
        for (int i = 0; i < N; ++i) { y[i] = Z(0, i); acor[i] = 0.0; }
      } else if (outcome >= 2) {
        retract();
        ++ncf; ++ncfn;
        if (outcome == 3 || ncf >= MXNCF || fabs(h) <= 100.0 * UROUND * fabs(t)) {
          fail_cell(CONV);
        } else {
          force_setup = true;
          etamax = 1.0;
          rescale(ETACF);
          phase = STEP;
        }
      } else if (outcome == 1) {
        const double acnrm2 = (m == 0) ? del2 : wms(acor);
        const double dsm2 = acnrm2 * (tq2 * tq2);  // squared local error estimate
        if (!(dsm2 <= 1.0)) {
          // ---- local error test failed ----
          retract();
          ++nef; ++netf;
          if (nef >= MXNEF || !isfinite(dsm2)) {
            fail_cell(isfinite(dsm2) ? ERRTEST : NONFINITE);
          } else {
            etamax = 1.0;
            if (nef <= MXNEF1) {
              double e = 1.0 / (pgb_pow64((BIAS2 * BIAS2) * dsm2, 0.5 * inv_int(q + 1)) + ADDON);
              e = fmax(ETAMIN, e);
              if (nef >= SMALL_NEF) e = fmin(e, ETAMXF);
              rescale(e);
              phase = STEP;
            } else if (q > 1) {
              adjust_order(-1);
              --q;
              qwait = q + 1;
              rescale(ETAMIN);
              phase = STEP;
            } else {
              rescale(ETAMIN);
              qwait = 10;
              phase = RESETD;
            }
            if (phase != NEED && fabs(h) <= 100.0 * UROUND * fabs(t)) fail_cell(HSMALL);
          }
        } else {
          // ---- step accepted: complete it ----
          ++nst;
          for (int i = q + 1; i >= 2; --i) TAU(i) = TAU(i - 1);
          TAU(1) = h;
          for (int j = 0; j <= q; ++j) {
            const double lj = LCO(j);
#pragma unroll
            for (int i = 0; i < N; ++i) Z(j, i) = fma(lj, acor[i], Z(j, i));
          }
          --qwait;
          if (qwait == 1 && q != qmax) {
#pragma unroll
            for (int i = 0; i < N; ++i) Z(QMAX + 1, i) = acor[i];
            tq5_saved = tq5;
          }
          if (fabs(t - tout) <= 100.0 * UROUND * (fabs(t) + fabs(h)) || t >= tout) {
            finish_cell();
          } else {
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
                  double zq[N];
#pragma unroll
                  for (int i = 0; i < N; ++i) zq[i] = Z(q, i);
                  const double ddn2 = wms(zq) * (tq1 * tq1);
                  etaqm1 = 1.0 / (pgb_pow64((BIAS1 * BIAS1) * ddn2, 0.5 * inv_int(q)) + ADDON);
                }
                if (q != qmax) {
                  const double hr = h / TAU(2);
                  double hrp = hr;
                  for (int k = 0; k < q; ++k) hrp *= hr;  // (h / tau2)^(q+1)
                  const double cquot = (tq5 / tq5_saved) * hrp;
                  double tv[N];
#pragma unroll
                  for (int i = 0; i < N; ++i) tv[i] = acor[i] - cquot * Z(QMAX + 1, i);
                  const double dup2 = wms(tv) * (tq3 * tq3);
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
                  for (int i = 0; i < N; ++i) Z(QMAX + 1, i) = acor[i];
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
            new_step = true;
            phase = STEP;
          }
        }
      }
    }
  }
#undef Z
#undef LCO
#undef TAU
#undef FRC
#undef LU
#undef PIV
#undef XS
}

}  // namespace pgb

#endif  // PGB_BDF_KERNEL_CUH
