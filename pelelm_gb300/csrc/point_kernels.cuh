// Pointwise kernels next to the reactor: instantaneous production rates
// (reactionRateRhoY, Source/PeleLM_K.H:54-98), T from (rho h, Y) (getTfromHY,
// Source/PeleLM_K.H:508-529 / RhoH_to_Temp, Source/PeleLM.cpp:8201-8287) and the null reactor
// (forcing only, the ReactorNull test double).
#ifndef PGB_POINT_KERNELS_CUH
#define PGB_POINT_KERNELS_CUH

#include "mech_common.cuh"
#include "mech_tables.cuh"
#include "reactor_types.cuh"

namespace pgb {

struct PointParams {
  int lo0, lo1, lo2, len0, len1, len2;
  ArrDev rY, rE, T, out;
  MaskDev mask;
  double tmin, tmax;
};

__device__ __forceinline__ double& arr_at(const ArrDev& a, int i, int j, int k, int n) {
  return a.p[(long long)(i - a.begin0) + (long long)(j - a.begin1) * a.jstride +
             (long long)(k - a.begin2) * a.kstride + (long long)n * a.nstride];
}

// Newton on h(T) = htarget [erg/g] with steps limited to 100 K and T clipped to [tmin, tmax]
// (the same iteration the CPU oracle uses).
template <class M>
__device__ __forceinline__ double hy2t_newton(double htarget, const double* Y, double T,
                                              double tmin, double tmax) {
  if (!(T > tmin && T < tmax)) T = 1000.0;
  for (int it = 0; it < 50; ++it) {
    double hh, cp;
    M::h_cp_mix(T, Y, hh, cp);
    double dT = (htarget - hh) / cp;
    dT = fmax(-100.0, fmin(100.0, dT));
    T = fmax(tmin, fmin(tmax, T + dT));
    if (fabs(dT) < 1e-10 * T) break;
  }
  return T;
}

template <class M>
__global__ void rates_kernel(const PointParams p) {
  const long long n = (long long)p.len0 * p.len1 * p.len2;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int i = p.lo0 + (int)(c % p.len0);
  const int j = p.lo1 + (int)((c / p.len0) % p.len1);
  const int k = p.lo2 + (int)(c / ((long long)p.len0 * p.len1));
  if (p.mask.p) {
    const int mv = p.mask.p[(long long)(i - p.mask.begin0) + (long long)(j - p.mask.begin1) * p.mask.jstride +
                            (long long)(k - p.mask.begin2) * p.mask.kstride];
    if (mv < 0) {
      for (int s = 0; s < M::NS; ++s) arr_at(p.out, i, j, k, s) = 0.0;
      return;
    }
  }
  double Y[M::NS], C[M::NS], wd[M::NS];
  double rho = 0.0;
#pragma unroll
  for (int s = 0; s < M::NS; ++s) { Y[s] = arr_at(p.rY, i, j, k, s); rho += Y[s]; }
  const double inv_rho = 1.0 / rho;
#pragma unroll
  for (int s = 0; s < M::NS; ++s) Y[s] *= inv_rho;
  // MKS -> CGS: h [J/kg] * 1e4 = erg/g ; rho [kg/m^3] * 1e-3 = g/cm^3
  const double T = hy2t_newton<M>(arr_at(p.rE, i, j, k, 0) * inv_rho * 1.0e4, Y, arr_at(p.T, i, j, k, 0),
                                  90.0, 5000.0);
  const double rho_cgs = rho * 1.0e-3;
#pragma unroll
  for (int s = 0; s < M::NS; ++s) C[s] = rho_cgs * Y[s] / M::W(s);
  M::wdot(T, C, wd);
#pragma unroll
  for (int s = 0; s < M::NS; ++s) arr_at(p.out, i, j, k, s) = wd[s] * M::W(s) * 1000.0;  // g/cm^3/s -> kg/m^3/s
}

template <class M>
__global__ void h2t_kernel(const PointParams p) {
  const long long n = (long long)p.len0 * p.len1 * p.len2;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int i = p.lo0 + (int)(c % p.len0);
  const int j = p.lo1 + (int)((c / p.len0) % p.len1);
  const int k = p.lo2 + (int)(c / ((long long)p.len0 * p.len1));
  double Y[M::NS];
  double rho = 0.0;
#pragma unroll
  for (int s = 0; s < M::NS; ++s) { Y[s] = arr_at(p.rY, i, j, k, s); rho += Y[s]; }
  const double inv_rho = 1.0 / rho;
#pragma unroll
  for (int s = 0; s < M::NS; ++s) Y[s] *= inv_rho;
  double& T = arr_at(p.T, i, j, k, 0);
  T = hy2t_newton<M>(arr_at(p.rE, i, j, k, 0) * inv_rho * 1.0e4, Y, T, p.tmin, p.tmax);
}

// Heat release rate -sum_k rhoYdot_k h_k(T) [W/m^3] from T and the MKS reaction rates
// rhoYdot [kg/m^3/s] (p.rY), h_k from the NASA-7 tables (erg/g, times 1e-4 -> J/kg); the
// per-cell work of the HeatRelease derive (Source/PeleLM_derive.cpp:627-650).
template <class M>
__global__ void heat_release_kernel(const PointParams p) {
  using Tab = typename M::TabG;
  const long long n = (long long)p.len0 * p.len1 * p.len2;
  const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= n) return;
  const int i = p.lo0 + (int)(c % p.len0);
  const int j = p.lo1 + (int)((c / p.len0) % p.len1);
  const int k = p.lo2 + (int)(c / ((long long)p.len0 * p.len1));
  const double T = arr_at(p.T, i, j, k, 0);
  const double invT = 1.0 / T;
  double hr = 0.0;
  for (int s = 0; s < M::NS; ++s) {
    const TabSpecies<double>& sp = Tab::template sp<double>(s);
    const double* hc = T < sp.Tmid ? sp.hlo : sp.hhi;
    const double hRT = fma(T, fma(T, fma(T, fma(T, hc[4], hc[3]), hc[2]), hc[1]), fma(hc[5], invT, hc[0]));
    const double h_mks = hRT * kRerg * T * sp.invW * 1.0e-4;  // erg/g -> J/kg
    hr = fma(-arr_at(p.rY, i, j, k, s), h_mks, hr);
  }
  arr_at(p.out, i, j, k, 0) = hr;
}

// ReactorNull: rhoY += dt F, rho h += dt F_h, T from the new (h, Y), FC = 0 (CGS, in place).
template <class M>
__global__ void null_reactor_kernel(const ReactParams P) {
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < P.ncell;
       c += (long long)gridDim.x * blockDim.x) {
    int lo = 0, hi = P.nbox - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (P.boxes[mid].cell_offset <= c) lo = mid; else hi = mid - 1;
    }
    const BoxDev& B = P.boxes[lo];
    long long r = c - B.cell_offset;
    const int i = B.lo0 + (int)(r % B.len0);
    r /= B.len0;
    const int j = B.lo1 + (int)(r % B.len1);
    const int k = B.lo2 + (int)(r / B.len1);
    if (B.mask.p) {
      const int mv = B.mask.p[(long long)(i - B.mask.begin0) + (long long)(j - B.mask.begin1) * B.mask.jstride +
                              (long long)(k - B.mask.begin2) * B.mask.kstride];
      if (mv < 0) {
        arr_at(B.FC, i, j, k, 0) = 0.0;
        if (B.IR.p)
          for (int s = 0; s < M::NS; ++s) arr_at(B.IR, i, j, k, s) = -arr_at(B.rYsrc, i, j, k, s);
        continue;
      }
    }
    double Y[M::NS];
    double rho = 0.0;
#pragma unroll
    for (int s = 0; s < M::NS; ++s) {
      double& v = arr_at(B.rY, i, j, k, s);
      const double vn = fma(P.dt, arr_at(B.rYsrc, i, j, k, s) * B.sY_in, v * B.sY_in);  // CGS
      const double vo = __dmul_rn(vn, B.sY_out);
      if (B.IR.p)
        arr_at(B.IR, i, j, k, s) = __dsub_rn(__dmul_rn(-__dsub_rn(v, vo), 1.0 / P.dt), arr_at(B.rYsrc, i, j, k, s));
      v = vo;
      Y[s] = vn;
      rho += vn;
    }
    double& rE = arr_at(B.rE, i, j, k, 0);
    const double rEn = fma(P.dt, arr_at(B.rEsrc, i, j, k, 0) * B.sE_in, rE * B.sE_in);  // CGS
    rE = rEn * B.sE_out;
    const double inv_rho = 1.0 / rho;
#pragma unroll
    for (int s = 0; s < M::NS; ++s) Y[s] *= inv_rho;
    double& T = arr_at(B.T, i, j, k, 0);
    T = hy2t_newton<M>(rEn * inv_rho, Y, T, 90.0, 5000.0);
    arr_at(B.FC, i, j, k, 0) = 0.0;
  }
}

}  // namespace pgb

#endif  // PGB_POINT_KERNELS_CUH
