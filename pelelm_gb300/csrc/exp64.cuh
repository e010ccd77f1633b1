// Table-driven FP64 exponential (method of Tang, ACM TOMS 15(2) 1989, 64-entry variant).
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

__device__ __constant__ static const double kExp64Table[64] = PGB_EXP64_TABLE;

__device__ __forceinline__ double pgb_exp64(double x) {
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
  const double s = kExp64Table[j];
  const double v = fma(s, p, s);
  const int hi = __double2hiint(v) + (m << 20);
  double res = __hiloint2double(hi, __double2loint(v));
  res = (m < -1021) ? 0.0 : res;
  res = (m > 1023) ? __longlong_as_double(0x7ff0000000000000LL) : res;
  return res;
}

}  // namespace pgb

#endif  // PGB_EXP64_CUH
