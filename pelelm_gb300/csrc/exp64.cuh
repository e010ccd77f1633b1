// Table-driven FP64 exponential and logarithm.
//
// Exponential: method of Tang, ACM TOMS 15(2) 1989, 64-entry variant.
//
//   x = N ln2/64 + r,  N = round(x 64/ln2),  |r| <= ln2/128
//   exp(x) = 2^(N>>6) * T[N&63] * (1 + p(r)),  T[j] = 2^(j/64),
//   p(r) = r + r^2/2 + r^3/6 + r^4/24 + r^5/120 (truncation < 4e-17 on |r| <= ln2/128).
//
// Ten FP64 pipe instructions: the rounding of x*64/ln2 uses the 1.5*2^52 shift trick, the
// reduction is Cody-Waite with an exact N*L1 product, and the final 2^m scaling is an integer
// add on the exponent field (integer pipe). Results below 2^-1021 flush to 0 and above 2^1023
// saturate to +inf; the rates evaluated with it never approach either bound.
#ifndef PGB_EXP64_CUH
#define PGB_EXP64_CUH

#include <cuda_runtime.h>

#include "gen/exp64_table.cuh"

namespace pgb {

// Tables in global memory, read through L1: lanes look up different entries, which the
// constant cache would serialize.
__device__ static const double kExp64Table[64] = PGB_EXP64_TABLE;

// Both functions are out of line (one copy per translation unit): the reactor kernels call
// them from many sites, and inlined copies filled the instruction cache, which limits these
// kernels (measured on GB300: the lane-group, warp and per-thread BDF kernels gained 9-26 % from
// the call; the throughput-bound rate kernel is unchanged).
static __device__ __noinline__ double pgb_exp64(double x) {
  constexpr double kShift = 6755399441055744.0;  // 1.5 * 2^52
  const double t = fma(x, PGB_EXP64_INV_LN2_64, kShift);
  const int n = __double2loint(t);
  const double nd = t - kShift;
  double r = fma(nd, -PGB_EXP64_L1, x);
  r = fma(nd, -PGB_EXP64_L2, r);
  const double r2 = r * r;
  double p = fma(r, fma(r, fma(r, 1.0 / 120.0, 1.0 / 24.0), 1.0 / 6.0), 0.5);
  p = fma(r2, p, r);
  const int j = n & 63;
  const int m = n >> 6;
  const double s = __ldg(&kExp64Table[j]);
  const double v = fma(s, p, s);
  const int hi = __double2hiint(v) + (m << 20);
  double res = __hiloint2double(hi, __double2loint(v));
  res = (m < -1021) ? 0.0 : res;
  res = (m > 1023) ? __longlong_as_double(0x7ff0000000000000LL) : res;
  return res;
}

// Logarithm: method of Tang, ACM TOMS 16(4) 1990, 64 breakpoints c_j = 1 + (j + 1/2)/64:
//   x = 2^e m (m in [1, 2)),  j = top six mantissa bits,  r = m / c_j - 1 in (-1/128, 1/128)
//   log x = e ln2 + log c_j + log1p(r),  log1p(r) = r - r^2/2 + ... + r^7/7 (truncation < 2e-17).
// Eleven FP64 pipe instructions (r through one FMA with a tabulated 1/c_j; the exponent and
// table index come from integer ops). Defined for positive normal x, the only arguments the
// rate code passes (temperatures, clipped reduced pressures, Troe centring factors).
__device__ static const double kLog64InvC[64] = PGB_LOG64_INVC;
__device__ static const double kLog64LogC[64] = PGB_LOG64_LOGC;

static __device__ __noinline__ double pgb_log64(double x) {
  const int hi = __double2hiint(x);
  const int lo = __double2loint(x);
  const int e = ((hi >> 20) & 0x7ff) - 1023;
  const int j = (hi >> 14) & 63;
  const double m = __hiloint2double((hi & 0x000fffff) | 0x3ff00000, lo);
  const double r = fma(m, __ldg(&kLog64InvC[j]), -1.0);
  const double r2 = r * r;
  double p = fma(r, fma(r, fma(r, fma(r, fma(r, 1.0 / 7.0, -1.0 / 6.0), 0.2), -0.25), 1.0 / 3.0), -0.5);
  p = fma(r2, p, r);
  const double ed = (double)e;
  return fma(ed, PGB_LOG64_LN2_HI, __ldg(&kLog64LogC[j]) + fma(ed, PGB_LOG64_LN2_LO, p));
}

// x^a for x > 0 through the two functions above (step-size heuristics).
__device__ __forceinline__ double pgb_pow64(double x, double a) { return pgb_exp64(a * pgb_log64(x)); }

}  // namespace pgb

#endif  // PGB_EXP64_CUH
