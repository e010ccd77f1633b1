// Persistent, work-stealing BDF reactor kernel with one cell per group of G lanes (32 / G cells
// per warp): the default for drm19-sized mechanisms (21 species, 84 reactions, N = 22).
//
// Same contract and algorithm as bdf_kernel.cuh and bdf_warp_kernel.cuh (the PelePhysics reactor
// called at Source/PeleLM.cpp:5752; CVODE-class fixed-leading-coefficient variable-order
// Nordsieck BDF, modified Newton with analytic Jacobian and dense partial-pivot LU, CVODE's
// documented step/order heuristics; its CPU statement is oracle/bdf_oracle.cpp).
//
// Why groups on GB300: an FP64 warp instruction occupies the FP64 pipe for the same time whatever
// its active mask, so FP64 work should fill lanes with different cells. A warp per cell leaves
// the scalar step logic (coefficients, error test, step and order selection: about half of the
// FP64 instructions for drm19) on one useful lane in 32 and rounds 84 reactions up to 96 lane
// slots; a thread per cell cannot hold a 22-unknown cell's state in registers and shared memory
// at useful occupancy. A group of G lanes per cell runs the scalar logic for 32 / G cells per
// instruction, spreads reactions and species over G lanes, and keeps each lane's share of the
// state vectors (ceil(N / G) elements) in registers.
//
//  * every group runs the flattened state machine of bdf_kernel.cuh: each pass evaluates one
//    FP64 right-hand side per active cell (group-parallel: species, then reactions, then a
//    species-major gather; group sums by xor shuffles inside the group's lane mask);
//  * Jacobian and LU (type JR: FP32 in mixed precision) are built one cell at a time by the
//    whole warp (warp_setup of bdf_warp_kernel.cuh, the same arithmetic as the warp mapping)
//    into the cell's matrix in shared memory; the triangular solves run per group (rows over
//    the group's lanes), the same operations in the same order as the warp mapping's solve;
//  * per cell in shared memory: Nordsieck history (+ saved correction), forcing, l and tau,
//    the matrix and its pivots; per warp one region that holds the cells' RHS scratch
//    (concentrations, g/RT, rates of progress) during the RHS and the Jacobian scratch
//    (per-reaction partials, NASA-7 terms) during the setups;
//  * a group whose cell is done takes the next cell index from the global queue (one atomic
//    per warp for all groups that need a cell: work stealing across all boxes);
//  * with a retry list (mixed precision), a failed cell is listed and left untouched for the
//    FP64 pass that follows on the same stream.
#ifndef PGB_BDF_GROUP_KERNEL_CUH
#define PGB_BDF_GROUP_KERNEL_CUH

#include "bdf_warp_kernel.cuh"

namespace pgb {

// Bytes of shared memory per cell (state that lives across passes), per cell of RHS scratch
// (concentrations, g/RT, rates of progress: live only inside group_rhs) and per warp. The RHS
// scratch of the warp's cells and the Jacobian scratch of the cooperative setup share one region:
// every pass evaluates the right-hand sides first and runs the setups after them, never both at
// once, and 3.3 KB less per warp (drm19) leaves room for more cells or more L1 for the tables.
template <class M, class JR>
__host__ __device__ constexpr int gbdf_cell_bytes() {
  constexpr int N = M::N;
  constexpr int nd = (QMAX + 2) * N + N + (QMAX + 1) + (QMAX + 2);
  constexpr int nj = N * (N + 1) + N;
  return (nd * 8 + nj * (int)sizeof(JR) + N * 4 + 15) / 16 * 16;
}
template <class M>
__host__ __device__ constexpr int gbdf_rhs_bytes() {
  return (2 * M::NS + M::NR) * 8;
}
template <class M, class JR>
__host__ __device__ constexpr int gbdf_setup_bytes() {
  constexpr int N = M::N, NS = M::NS, NR = M::NR;
  return N * 8 + (N + wbdf::RXW * NR + 4 * NS) * (int)sizeof(JR);
}
template <class M, class JR, int G>
__host__ __device__ constexpr int gbdf_shared_scratch_bytes() {
  constexpr int a = (32 / G) * gbdf_rhs_bytes<M>(), b = gbdf_setup_bytes<M, JR>();
  return ((a > b ? a : b) + 15) / 16 * 16;
}
template <class M, class JR, int G>
__host__ __device__ constexpr int gbdf_smem_per_warp() {
  return (32 / G) * gbdf_cell_bytes<M, JR>() + gbdf_shared_scratch_bytes<M, JR, G>();
}

// The group-distributed part of a length-N vector (element i in sub-lane i % G, slot i / G).
template <class M, int G>
struct GVec {
  double v[(M::N + G - 1) / G];
};

template <int G>
__device__ __forceinline__ unsigned group_mask() {
  if constexpr (G == 32) {
    return 0xffffffffu;
  } else {
    const int lane = threadIdx.x & 31;
    return ((1u << G) - 1u) << (lane - lane % G);
  }
}
template <int G>
__device__ __forceinline__ double group_sum(double v, unsigned gm) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(gm, v, o);
  return v;
}
template <int G>
__device__ __forceinline__ double group_max(double v, unsigned gm) {
#pragma unroll
  for (int o = G / 2; o > 0; o >>= 1) v = fmax(v, __shfl_xor_sync(gm, v, o));
  return v;
}

// Right-hand side f = [W_k wdot_k + F_k, dT/dt] at y for one cell, its group of G lanes
// cooperating (the equations of warp_rhs with G lanes in place of 32). Inlined: the kernel calls
// it from one place, so inlining adds no copy and removes the call's register save and restore
// (measured: no spills left, +5 %).
template <class M, int G>
__device__ __forceinline__ GVec<M, G> group_rhs(const GVec<M, G> yv, double* CS, double* GS, double* QS,
                                             const double* FRC) {
  using Tab = typename M::TabG;
  constexpr int N = M::N, NS = M::NS, NR = M::NR;
  constexpr int R = (N + G - 1) / G;
  const int lane = threadIdx.x & 31, sub = lane % G, gbase = lane - sub;
  const unsigned gm = group_mask<G>();
  auto idx = [&](int r) { return sub + G * r; };
  const double (&y)[R] = yv.v;
  GVec<M, G> fv;
  double (&f)[R] = fv.v;
  const double T = __shfl_sync(gm, y[NS / G], gbase + NS % G);
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
  const double Ctot = group_sum<G>(c_loc, gm);
  __syncwarp(gm);
  for (int j = sub; j < NR; j += G) {
    QS[j] = rate_of_progress<Tab>(j, T, invT, lnT, lnP0RT, Ctot, CS, GS);
  }
  __syncwarp(gm);
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
  hs = group_sum<G>(hs, gm);
  rcp = group_sum<G>(rcp, gm);
  const double fT = fma(-hs, kRerg * T, FRC[NS]) / (rcp * kRerg);
#pragma unroll
  for (int r = 0; r < R; ++r)
    if (idx(r) == NS) f[r] = fT;
  __syncwarp(gm);  // CS/GS/QS are reused by the next evaluation
  return fv;
}

template <class M, class JR, int G, int WPB>
__global__ void __launch_bounds__(WPB * 32, 1) bdf_group_kernel(const ReactParams P) {
  using namespace bdf;
  using Tab = typename M::TabG;
  static_assert(G == 4 || G == 8 || G == 16 || G == 32, "group size must divide the warp");
  constexpr int N = M::N, NS = M::NS, NR = M::NR;
  constexpr int R = (N + G - 1) / G;  // vector elements per lane
  constexpr int LDA = N + 1;          // padded matrix row
  constexpr int CPW = 32 / G;         // cells per warp
  constexpr bool MIXED = sizeof(JR) == sizeof(float);
  constexpr int RW = (N + 31) / 32;   // slots of the warp-wide setup vector
  extern __shared__ __align__(16) unsigned char gsmem[];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int sub = lane % G, grp = lane / G, gbase = lane - sub;
  const unsigned gm = group_mask<G>();
  unsigned char* wbase = gsmem + (size_t)wid * gbdf_smem_per_warp<M, JR, G>();
  auto cell_base = [&](int g) { return wbase + (size_t)g * gbdf_cell_bytes<M, JR>(); };
  unsigned char* const wscratch = cell_base(CPW);  // RHS scratch of the cells | setup scratch
  struct CellMem {
    double *Z, *FRC, *CS, *GS, *QS, *LC, *TAU;
    JR *A, *XS;
    int* PIV;
  };
  auto cell_mem = [&](int g) {
    CellMem c;
    c.Z = reinterpret_cast<double*>(cell_base(g));  // [(QMAX+2)][N]; column QMAX+1: saved acor
    c.FRC = c.Z + (QMAX + 2) * N;                   // [N] forcing (rhoY, then rho h)
    c.CS = reinterpret_cast<double*>(wscratch + (size_t)g * gbdf_rhs_bytes<M>());  // [NS] concentrations
    c.GS = c.CS + NS;                               // [NS] g/RT
    c.QS = c.GS + NS;                               // [NR] rates of progress
    c.LC = c.FRC + N;                               // [QMAX+1] l coefficients
    c.TAU = c.LC + (QMAX + 1);                      // [QMAX+2] step history
    c.A = reinterpret_cast<JR*>(c.TAU + (QMAX + 2));  // [N][LDA] matrix, then its LU
    c.XS = c.A + N * LDA;                           // [N] solve vector
    c.PIV = reinterpret_cast<int*>(c.XS + N);       // [N] pivots
    return c;
  };
  const CellMem C = cell_mem(grp);
  double* const YS = reinterpret_cast<double*>(wscratch);         // [N] setup input staging
  JR* const WXS = reinterpret_cast<JR*>(YS + N);                  // [N] setup concentrations
  JR* const WRX = WXS + N;                                        // [NR][RXW] Jacobian partials
  JR* const WTH = WRX + wbdf::RXW * NR;                           // [4][NS] NASA-7 terms

  const long long ncell = P.ncell_dev ? (long long)*P.ncell_dev : P.ncell;
  const int qmax = max(1, min(P.max_order, QMAX));
  const double tout = P.dt;
  auto idx = [&](int r) { return sub + G * r; };
  auto Z = [&](int j, int r) -> double& { return C.Z[j * N + idx(r)]; };

  // ---- per-group state (scalars replicated in the group's lanes; vectors distributed) ----
  int phase = NEED;
  long long cell = -1;
  int box = 0, ci = 0, cj = 0, ck = 0;
  double y[R], acor[R], ewt[R];
  double t = 0.0, h = 0.0, hscale = 0.0, etamax = ETAMX1, eta = 1.0;
  double gamma = 0.0, gammap = 0.0, gamrat = 1.0, crate2 = 1.0, rl1 = 1.0;
  double tq1 = 1.0, tq2 = 1.0, tq3 = 1.0, tq5 = 1.0, tq5_saved = 1.0, inv_tq4_sq = 1.0;
  double del2 = 0.0, delp2 = 0.0, hg = 0.0, hub = 0.0, hlb = 0.0, rE0 = 0.0;
  int q = 1, qwait = 2, nef = 0, ncf = 0, m = 0, hin_count = 0, status = OK;
  int nst = 0, nfe = 0, nje = 0, nstlp = 0, netf = 0, ncfn = 0;  // bounded by ode.max_steps
  bool new_step = true, need_setup = true, force_setup = true, jcur = false, setup_ok = true;
#pragma unroll
  for (int r = 0; r < R; ++r) { y[r] = 0.0; acor[r] = 0.0; ewt[r] = 1.0; }

  auto wms = [&](const double (&v)[R]) -> double {  // squared WRMS norm
    double s = 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < N) { const double x = v[r] * ewt[r]; s = fma(x, x, s); }
    return group_sum<G>(s, gm) * (1.0 / N);
  };
  auto set_ewt = [&]() {
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < N) {
        const double d = fma(P.rtol, fabs(Z(0, r)), P.atol[idx(r)]);
        ewt[r] = MIXED ? recip_fast(d) : 1.0 / d;
      }
  };
  auto rescale = [&](double e) {
    double fac = e;
    for (int j = 1; j <= q; ++j) {
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (idx(r) < N) Z(j, r) *= fac;
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
          if (idx(r) < N) Z(j - 1, r) += Z(j, r);
  };
  auto retract = [&]() {
    t -= h;
    for (int k = 1; k <= q; ++k)
      for (int j = q; j >= k; --j)
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (idx(r) < N) Z(j - 1, r) -= Z(j, r);
  };
  auto tau = [&](int j) -> double { return C.TAU[j]; };
  // l coefficients and error constants (the arithmetic of bdf_kernel.cuh's set_coeffs); l is
  // computed in registers by every lane of the group and stored once
  auto set_coeffs = [&]() {
    double l[QMAX + 1];
#pragma unroll
    for (int i = 0; i <= QMAX; ++i) l[i] = 0.0;
    l[0] = 1.0;
    double alpha0 = 0.0;
    for (int j = 1; j <= q; ++j) alpha0 -= inv_int(j);
    double hsum = h, sum_xi_inv = 0.0;
    for (int i = 1; i <= q - 1; ++i) {
      if (i > 1) hsum += tau(i - 1);
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
    if (q > 1) hsum += tau(q - 1);
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
        const double Cq = xistar_inv / lq;
        const double A3 = alpha0 + inv_int(q);
        const double A4 = alpha0_hat + xiq_inv;
        tq1 = fabs(Cq * (1.0 - A4 + A3) / A3);
      } else {
        tq1 = 1.0;
      }
      const double xiq1_inv = h / (hsum + tau(q));
      const double A5 = alpha0 - inv_int(q + 1);
      const double A6 = alpha0_hat - xiq1_inv;
      const double Cpp = (1.0 - A6 + A5) / A2;
      tq3 = fabs(Cpp / (xiq1_inv * (q + 2) * A5));
    }
    inv_tq4_sq = (tq2 * (1.0 / NLSCOEF)) * (tq2 * (1.0 / NLSCOEF));
    rl1 = 1.0 / l[1];
    __syncwarp(gm);
    for (int e = sub; e <= QMAX; e += G) {
      double v = 0.0;
#pragma unroll
      for (int k = 0; k <= QMAX; ++k) if (k == e) v = l[k];
      C.LC[e] = v;
    }
    __syncwarp(gm);
  };
  auto adjust_order = [&](int dq) {
    double w[QMAX + 2];
#pragma unroll
    for (int i = 0; i < QMAX + 2; ++i) w[i] = 0.0;
    w[2] = 1.0;
    if (dq > 0) {
      double alpha0 = 0.0, alpha1 = 0.0, prod = 1.0, hsum = 0.0;
      for (int j = 1; j <= q; ++j) {
        hsum += tau(j);
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
        if (idx(r) < N) Z(q + 1, r) = A1 * Z(QMAX + 1, r);
#pragma unroll
      for (int j = 2; j <= QMAX; ++j)
        if (j <= q)
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (idx(r) < N) Z(j, r) = fma(w[j], Z(q + 1, r), Z(j, r));
    } else {
      double hsum = 0.0;
      for (int j = 1; j <= q - 2; ++j) {
        hsum += tau(j);
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
            if (idx(r) < N) Z(j, r) = fma(-w[j], Z(q, r), Z(j, r));
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (idx(r) < N) Z(q, r) = 0.0;
    }
  };
  // (I - gamma J) x = b with the cell's factors: rows over the group's lanes, the operations and
  // their order of the warp mapping's solve
  auto solve = [&](double (&b)[R]) {
    JR* XS = C.XS;
    const JR* A = C.A;
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < N) XS[idx(r)] = (JR)b[r];
    __syncwarp(gm);
#pragma unroll 1
    for (int k = 0; k < N; ++k) {
      const int p = C.PIV[k];
      if (p != k && sub == 0) { const JR tmp = XS[k]; XS[k] = XS[p]; XS[p] = tmp; }
      __syncwarp(gm);
      const JR bk = XS[k];
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = idx(r);
        if (i > k && i < N) XS[i] -= A[i * LDA + k] * bk;
      }
      __syncwarp(gm);
    }
#pragma unroll 1
    for (int k = N - 1; k >= 0; --k) {
      const JR xk = XS[k] * A[k * LDA + k];
      __syncwarp(gm);
      if (sub == 0) XS[k] = xk;
#pragma unroll
      for (int r = 0; r < R; ++r) {
        const int i = idx(r);
        if (i < k) XS[i] -= A[i * LDA + k] * xk;
      }
      __syncwarp(gm);
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < N) b[r] = (double)XS[idx(r)];
    __syncwarp(gm);
  };
  // ---- cell I/O ----
  auto elem = [&](const ArrDev& a, int n) -> double& {
    return a.p[(long long)(ci - a.begin0) + (long long)(cj - a.begin1) * a.jstride +
               (long long)(ck - a.begin2) * a.kstride + (long long)n * a.nstride];
  };
  auto add_stats = [&](bool retried) {
    if (sub != 0) return;
    ReactStats* S = P.stats;
    atomicAdd(&S->nst, (unsigned long long)nst);
    atomicAdd(&S->nfe, (unsigned long long)nfe);
    atomicAdd(&S->nje, (unsigned long long)nje);
    atomicAdd(&S->netf, (unsigned long long)netf);
    atomicAdd(&S->ncfn, (unsigned long long)ncfn);
    if (retried) {
      atomicAdd(&S->nretry, 1ull);
      return;
    }
    if (status != OK) atomicAdd(&S->nfail, 1ull);
    atomicMax(&S->max_nst, (unsigned long long)nst);
    const int bin = min(15, 31 - __clz(max(nst, 1)));
    atomicAdd(&S->hist[bin], 1ull);
  };
  auto finish_cell = [&]() {
    const BoxDev& B = P.boxes[box];
    if (status != OK && P.retry_list) {  // hand the cell to the retry pass, arrays untouched
      if (sub == 0) P.retry_list[atomicAdd(P.retry_count, 1ull)] = cell;
      add_stats(true);
      phase = NEED;
      return;
    }
    // rho h(t) = rho h0 + F_h t ; T from (h, Y) by Newton with the integrated T as guess
    const double rE = fma(tout, C.FRC[NS], rE0);
    double rho_l = 0.0;
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < NS) rho_l += Z(0, r);
    const double inv_rho = 1.0 / group_sum<G>(rho_l, gm);
    const double htarget = rE * inv_rho;
    double Tn = C.Z[NS];
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
          const double Yk = Z(0, r) * inv_rho;
          hl = fma(Yk * s.invW, hRT * kRerg * Tn, hl);
          cl = fma(Yk * s.invW, cpR * kRerg, cl);
        }
      }
      const double hh = group_sum<G>(hl, gm), cp = group_sum<G>(cl, gm);
      double dT = (htarget - hh) / cp;
      dT = fmax(-100.0, fmin(100.0, dT));
      Tn = fmax(90.0, fmin(5000.0, Tn + dT));
      if (fabs(dT) < 1e-10 * Tn) break;
    }
#pragma unroll
    for (int r = 0; r < R; ++r)
      if (idx(r) < NS) {
        const double rYn = __dmul_rn(Z(0, r), B.sY_out);
        if (B.IR.p)  // separate roundings, as separate passes over arrays give
          elem(B.IR, idx(r)) = __dsub_rn(__dmul_rn(-__dsub_rn(elem(B.rY, idx(r)), rYn), 1.0 / tout),
                                         elem(B.rYsrc, idx(r)));
        elem(B.rY, idx(r)) = rYn;
      }
    if (sub == 0) {
      elem(B.T, 0) = Tn;
      elem(B.rE, 0) = rE * B.sE_out;
      elem(B.FC, 0) = (status == OK) ? (double)nfe : -(double)status;
    }
    add_stats(false);
    phase = NEED;
  };
  auto fail_cell = [&](int st) {
    status = st;
    phase = FINISH;
  };
  // loads flat cell c into the group; false for a covered cell (FC = 0, I_R = -F written)
  auto load_cell = [&](long long c) -> bool {
    int lo = 0, hi = P.nbox - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (P.boxes[mid].cell_offset <= c) lo = mid; else hi = mid - 1;
    }
    box = lo;
    const BoxDev& B = P.boxes[box];
    long long rr = c - B.cell_offset;
    ci = B.lo0 + (int)(rr % B.len0);
    rr /= B.len0;
    cj = B.lo1 + (int)(rr % B.len1);
    ck = B.lo2 + (int)(rr / B.len1);
    if (B.mask.p && B.mask.p[(long long)(ci - B.mask.begin0) + (long long)(cj - B.mask.begin1) * B.mask.jstride +
                             (long long)(ck - B.mask.begin2) * B.mask.kstride] < 0) {
      if (sub == 0) elem(B.FC, 0) = 0.0;
      if (B.IR.p)
        for (int k = sub; k < NS; k += G) elem(B.IR, k) = -elem(B.rYsrc, k);
      return false;
    }
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = idx(r);
      if (i < NS) { Z(0, r) = elem(B.rY, i) * B.sY_in; C.FRC[i] = elem(B.rYsrc, i) * B.sY_in; }
      else if (i == NS) { Z(0, r) = elem(B.T, 0); C.FRC[NS] = elem(B.rEsrc, 0) * B.sE_in; }
    }
    for (int e = sub; e < (QMAX + 1) * N; e += G) C.Z[N + e] = 0.0;  // columns 1..QMAX+1
    for (int e = sub; e < QMAX + 2; e += G) C.TAU[e] = 0.0;
    rE0 = elem(B.rE, 0) * B.sE_in;
    t = 0.0; h = 0.0; hscale = 0.0; etamax = ETAMX1; eta = 1.0;
    gamma = 0.0; gammap = 0.0; gamrat = 1.0; crate2 = 1.0; rl1 = 1.0;
    tq1 = tq2 = tq3 = tq5 = tq5_saved = inv_tq4_sq = 1.0;
    q = 1; qwait = 2; nef = 0; ncf = 0; m = 0; status = OK;
    nst = 0; nfe = 0; nje = 0; nstlp = 0; netf = 0; ncfn = 0;
    new_step = true; need_setup = true; force_setup = true; jcur = false;
    __syncwarp(gm);
    return true;
  };

  for (;;) {
    // ------------------------------------------------ (A) work stealing, one atomic per warp
    {
      const unsigned need = __ballot_sync(0xffffffffu, phase == NEED && sub == 0);
      if (need) {
        const int leader = __ffs(need) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(P.next_cell, (unsigned long long)__popc(need));
        base = __shfl_sync(0xffffffffu, base, leader);
        const long long c = (long long)base + __popc(need & ((1u << gbase) - 1u));
        if (phase == NEED) {
          if (c >= ncell) {
            phase = IDLE;
          } else {
            cell = P.cell_list ? P.cell_list[c] : c;
            if (load_cell(cell)) phase = START;  // covered cells stay NEED and refetch next pass
          }
        }
      }
      if (__all_sync(0xffffffffu, phase == IDLE)) break;
    }

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
        gamma = h * rl1;
        if (nst == 0) gammap = gamma;
        gamrat = (nst > 0) ? gamma / gammap : 1.0;
        need_setup = force_setup || nst == 0 || nst >= nstlp + MSBP || fabs(gamrat - 1.0) > DGMAX;
        force_setup = false;
        jcur = false;
        m = 0;
#pragma unroll
        for (int r = 0; r < R; ++r) { y[r] = idx(r) < N ? Z(0, r) : 0.0; acor[r] = 0.0; }
        phase = NEWTON;
      }
    } else if (phase == HIN) {
#pragma unroll
      for (int r = 0; r < R; ++r) y[r] = idx(r) < N ? fma(hg, Z(1, r), Z(0, r)) : 0.0;
    } else if (phase == START || phase == RESETD) {
#pragma unroll
      for (int r = 0; r < R; ++r) y[r] = idx(r) < N ? Z(0, r) : 0.0;
    }

    // ------------------------------------------------ (C) one FP64 RHS per active cell
    double f[R];
    const bool active = phase >= START;
    if (active) {
      GVec<M, G> yv;
#pragma unroll
      for (int r = 0; r < R; ++r) yv.v[r] = y[r];
      const GVec<M, G> fv = group_rhs<M, G>(yv, C.CS, C.GS, C.QS, C.FRC);
#pragma unroll
      for (int r = 0; r < R; ++r) f[r] = fv.v[r];
      ++nfe;
    } else {
#pragma unroll
      for (int r = 0; r < R; ++r) f[r] = 0.0;
    }

    // ------------------------------------------------ (E) Jacobian setups, one cell at a time
    // by the whole warp (cells that start a Newton iteration with a stale or missing matrix)
    __syncwarp();
    {
      unsigned todo = __ballot_sync(0xffffffffu, sub == 0 && phase == NEWTON && m == 0 && need_setup);
      while (todo) {
        const int g = (__ffs(todo) - 1) / G;
        todo &= todo - 1;
        if (grp == g) {
#pragma unroll
          for (int r = 0; r < R; ++r)
            if (idx(r) < N) YS[idx(r)] = y[r];
        }
        __syncwarp();
        WVec<M> yv;
#pragma unroll
        for (int s = 0; s < RW; ++s) {
          const int i = lane + 32 * s;
          yv.v[s] = i < N ? YS[i] : 0.0;
        }
        const double gam = __shfl_sync(0xffffffffu, gamma, g * G);
        const CellMem Cg = cell_mem(g);
        const bool ok = warp_setup<M, JR>(yv, gam, Cg.FRC, Cg.A, WXS, WRX, WTH, Cg.PIV);
        __syncwarp();
        if (grp == g) {
          setup_ok = ok;
          ++nje;
          gammap = gamma;
          gamrat = 1.0;
          crate2 = 1.0;
          nstlp = nst;
        }
      }
    }

    // ------------------------------------------------ (D) consume it
    if (phase == START) {
      // initial step size: difference-quotient estimate of y'' (bounded)
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (idx(r) < N) Z(1, r) = f[r];  // f0 parked in z[1] until h is known
      set_ewt();
      const double tround = UROUND * tout;
      hlb = 100.0 * tround;
      double hub_inv = 0.0;
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (idx(r) < N) hub_inv = fmax(hub_inv, fabs(f[r]) / fma(0.1, fabs(Z(0, r)), P.atol[idx(r)]));
      hub_inv = group_max<G>(hub_inv, gm);
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
        for (int r = 0; r < R; ++r)
          if (idx(r) < N) Z(1, r) *= h;
        q = 1; qwait = 2; etamax = ETAMX1;
        __syncwarp(gm);
        if (sub == 0) C.TAU[1] = h;
        new_step = true;
        phase = STEP;
      }
    } else if (phase == HIN) {
      double d[R];
#pragma unroll
      for (int r = 0; r < R; ++r) d[r] = idx(r) < N ? (f[r] - Z(1, r)) / hg : 0.0;
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
        for (int r = 0; r < R; ++r)
          if (idx(r) < N) Z(1, r) *= h;
        q = 1; qwait = 2; etamax = ETAMX1;
        __syncwarp(gm);
        if (sub == 0) C.TAU[1] = h;
        new_step = true;
        phase = STEP;
      }
    } else if (phase == RESETD) {
#pragma unroll
      for (int r = 0; r < R; ++r)
        if (idx(r) < N) Z(1, r) = h * f[r];
      phase = STEP;
    } else if (phase == NEWTON) {
      bool singular = false;
      if (m == 0 && need_setup) {
        singular = !setup_ok;
        need_setup = false;
        jcur = true;
      }
      int outcome = 0;  // 0 continue, 1 converged, 2 convergence failure, 3 singular matrix
      if (singular) {
        outcome = 3;
      } else {
        double b[R];
#pragma unroll
        for (int r = 0; r < R; ++r) b[r] = idx(r) < N ? fma(gamma, f[r], -fma(rl1, Z(1, r), acor[r])) : 0.0;
        solve(b);
        if (gamrat != 1.0) {
          const double s = 2.0 / (1.0 + gamrat);
#pragma unroll
          for (int r = 0; r < R; ++r) b[r] *= s;
        }
        del2 = wms(b);
#pragma unroll
        for (int r = 0; r < R; ++r)
          if (idx(r) < N) { acor[r] += b[r]; y[r] = Z(0, r) + acor[r]; }
        if (m > 0) crate2 = fmax((CRDOWN * CRDOWN) * crate2, del2 / delp2);
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
        for (int r = 0; r < R; ++r) { y[r] = idx(r) < N ? Z(0, r) : 0.0; acor[r] = 0.0; }
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
            if (phase != FINISH && fabs(h) <= 100.0 * UROUND * fabs(t)) fail_cell(HSMALL);
          }
        } else {
          // ---- step accepted: complete it ----
          ++nst;
          __syncwarp(gm);
          if (sub == 0) {
            for (int i = q + 1; i >= 2; --i) C.TAU[i] = C.TAU[i - 1];
            C.TAU[1] = h;
          }
          for (int j = 0; j <= q; ++j) {
            const double lj = C.LC[j];
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (idx(r) < N) Z(j, r) = fma(lj, acor[r], Z(j, r));
          }
          __syncwarp(gm);
          --qwait;
          if (qwait == 1 && q != qmax) {
#pragma unroll
            for (int r = 0; r < R; ++r)
              if (idx(r) < N) Z(QMAX + 1, r) = acor[r];
            tq5_saved = tq5;
          }
          if (fabs(t - tout) <= 100.0 * UROUND * (fabs(t) + fabs(h)) || t >= tout) {
            phase = FINISH;
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
                  double zq[R];
#pragma unroll
                  for (int r = 0; r < R; ++r) zq[r] = idx(r) < N ? Z(q, r) : 0.0;
                  const double ddn2 = wms(zq) * (tq1 * tq1);
                  etaqm1 = 1.0 / (pgb_pow64((BIAS1 * BIAS1) * ddn2, 0.5 * inv_int(q)) + ADDON);
                }
                if (q != qmax) {
                  const double hr = h / tau(2);
                  double hrp = hr;
                  for (int k = 0; k < q; ++k) hrp *= hr;  // (h / tau2)^(q+1)
                  const double cquot = (tq5 / tq5_saved) * hrp;
                  double tv[R];
#pragma unroll
                  for (int r = 0; r < R; ++r) tv[r] = idx(r) < N ? acor[r] - cquot * Z(QMAX + 1, r) : 0.0;
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
                  for (int r = 0; r < R; ++r)
                    if (idx(r) < N) Z(QMAX + 1, r) = acor[r];
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
    // ------------------------------------------------ (F) write back a finished cell
    if (phase == FINISH) finish_cell();
    __syncwarp();
  }
}

}  // namespace pgb

#endif  // PGB_BDF_GROUP_KERNEL_CUH
