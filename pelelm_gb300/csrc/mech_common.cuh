// Device math shared by the generated mechanism headers and the reactor kernels.
#ifndef PGB_MECH_COMMON_CUH
#define PGB_MECH_COMMON_CUH

#include <cuda_runtime.h>
#include <math.h>

#include "exp64.cuh"

namespace pgb {

// FP64 exponential / logarithm used by every rate evaluation.
__device__ __forceinline__ double pgb_exp(double x) { return pgb_exp64(x); }
__device__ __forceinline__ double pgb_log(double x) { return pgb_log64(x); }

// Precision-generic versions used by the Jacobian template. The FP32 path uses the
// hardware exponential / logarithm with the argument clamped to the finite FP32 range, so
// a rate coefficient outside that range saturates instead of turning into inf/NaN (the
// FP32 Jacobian only preconditions Newton; residuals stay FP64).
template <class R> __device__ __forceinline__ R pgb_expT(R x);
template <class R> __device__ __forceinline__ R pgb_logT(R x);

template <> __device__ __forceinline__ double pgb_expT<double>(double x) { return pgb_exp(x); }
template <> __device__ __forceinline__ double pgb_logT<double>(double x) { return pgb_log(x); }
template <> __device__ __forceinline__ float pgb_expT<float>(float x) {
  return __expf(fminf(fmaxf(x, -87.0f), 88.0f));
}
template <> __device__ __forceinline__ float pgb_logT<float>(float x) {
  return __logf(fmaxf(x, 1e-37f));
}

}  // namespace pgb

#endif  // PGB_MECH_COMMON_CUH
