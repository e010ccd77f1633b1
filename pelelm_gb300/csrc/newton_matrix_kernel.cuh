// Diagnostic kernels: the Newton matrix pieces of the BDF kernels for a batch of states, so a
// test can hold them against the oracle directly (the analytic Jacobian of
// Source/PeleLM.cpp:5752's CVODE reactor, cvode.solve_type = denseAJ_direct, and its dense
// solve). Each runs the production code:
//  * warp and lane-group kernels: one warp per cell; warp_setup without its factorization gives
//    J, warp_setup with it and warp_lu_solve give x solving (I - gamma J) x = b;
//  * cell-per-thread kernels: one thread per cell; the Jacobian call of their matrix setup
//    (the generated M::jac, or jac_table for table-driven mechanisms) gives J.
#ifndef PGB_NEWTON_MATRIX_KERNEL_CUH
#define PGB_NEWTON_MATRIX_KERNEL_CUH

#include "bdf_kernel.cuh"
#include "bdf_warp_kernel.cuh"

namespace pgb {

struct NewtonMatrixParams {
  long long ncell;
  const double* y;   // [ncell][N]  rhoY (CGS), then T
  const double* F;   // [ncell][NS] rhoY forcing (CGS)
  const double* Fh;  // [ncell]     rho h forcing (CGS)
  const double* b;   // [ncell][N]
  double gamma;
  double* J;         // [ncell][N][N] row-major, d ydot_i / d y_k
  double* x;         // [ncell][N]   NaN where the matrix is singular
};

// Shared bytes of one block (one warp): forcing, setup scratch, matrix, solve vector, pivots.
template <class M, class JR>
__host__ __device__ constexpr int newton_matrix_smem() {
  constexpr int N = M::N, NS = M::NS, NR = M::NR;
  return (N * 8 + 15) / 16 * 16 + ((wbdf::RXW * NR + 4 * NS) * (int)sizeof(JR) + 15) / 16 * 16 +
         ((N * (N + 1) + N) * (int)sizeof(JR) + 15) / 16 * 16 + N * 4;
}

template <class M, class JR>
__global__ void __launch_bounds__(32) newton_matrix_kernel(const NewtonMatrixParams P) {
  constexpr int N = M::N, NS = M::NS, NR = M::NR;
  constexpr int R = (N + 31) / 32, LDA = N + 1;
  extern __shared__ __align__(16) unsigned char nsmem[];
  const int lane = threadIdx.x & 31;
  double* FRC = reinterpret_cast<double*>(nsmem);
  JR* RX = reinterpret_cast<JR*>(nsmem + (N * 8 + 15) / 16 * 16);
  JR* TH = RX + wbdf::RXW * NR;
  JR* A = reinterpret_cast<JR*>(reinterpret_cast<unsigned char*>(RX) +
                                ((wbdf::RXW * NR + 4 * NS) * (int)sizeof(JR) + 15) / 16 * 16);
  JR* XS = A + N * LDA;
  int* PIV = reinterpret_cast<int*>(XS + N);
  for (long long c = blockIdx.x; c < P.ncell; c += gridDim.x) {
    WVec<M> yv;
    double b[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = lane + 32 * r;
      yv.v[r] = i < N ? P.y[c * N + i] : 0.0;
      b[r] = i < N ? P.b[c * N + i] : 0.0;
    }
    for (int i = lane; i < NS; i += 32) FRC[i] = P.F[c * NS + i];
    if (lane == 0) FRC[NS] = P.Fh[c];
    __syncwarp();
    warp_setup<M, JR, false>(yv, P.gamma, FRC, A, XS, RX, TH, PIV);
    __syncwarp();
    for (int e = lane; e < N * N; e += 32) {
      const int i = e / N, k = e - i * N;
      P.J[c * N * N + e] = (double)A[i * LDA + k];
    }
    __syncwarp();
    const bool ok = warp_setup<M, JR, true>(yv, P.gamma, FRC, A, XS, RX, TH, PIV);
    __syncwarp();
    if (ok) warp_lu_solve<M, JR>(A, PIV, XS, b);
#pragma unroll
    for (int r = 0; r < R; ++r) {
      const int i = lane + 32 * r;
      if (i < N) P.x[c * N + i] = ok ? b[r] : __longlong_as_double(0x7ff8000000000000LL);
    }
    __syncwarp();
  }
}

// Shared bytes of one 32-thread block of the per-thread variant: each thread's J and
// concentration scratch laid out [element][thread], as in the per-thread BDF kernel.
template <class M, class JR>
__host__ __device__ constexpr int newton_matrix_thread_smem() {
  return 32 * (M::N * M::N + M::N) * (int)sizeof(JR);
}

template <class M, class JR>
__global__ void __launch_bounds__(32) newton_matrix_thread_kernel(const NewtonMatrixParams P) {
  constexpr int N = M::N, NS = M::NS;
  extern __shared__ __align__(16) unsigned char tsmem[];
  JR* Jt = reinterpret_cast<JR*>(tsmem) + threadIdx.x;  // element (i, k) at (i N + k) 32
  JR* Ct = reinterpret_cast<JR*>(tsmem) + 32 * N * N + threadIdx.x;
  for (long long c = (long long)blockIdx.x * 32 + threadIdx.x; c < P.ncell; c += (long long)gridDim.x * 32) {
    double y[N];
#pragma unroll
    for (int i = 0; i < N; ++i) y[i] = P.y[c * N + i];
    const double* F = P.F + c * NS;
    LuAcc<JR> acc{Jt, N, 32};
    if constexpr (M::JAC_TABLE) {
      jac_table<typename M::Tab, JR>(y, [&](int k) -> double { return F[k]; }, P.Fh[c], acc,
                                     [&](int k) -> JR& { return Ct[k * 32]; });
    } else {
      double Fl[NS];
#pragma unroll
      for (int i = 0; i < NS; ++i) Fl[i] = F[i];
      M::template jac<JR>(y, Fl, P.Fh[c], acc);
    }
    for (int i = 0; i < N; ++i)
      for (int k = 0; k < N; ++k) P.J[c * N * N + i * N + k] = (double)acc(i, k);
    for (int i = 0; i < N; ++i) P.x[c * N + i] = __longlong_as_double(0x7ff8000000000000LL);
  }
}

}  // namespace pgb

#endif  // PGB_NEWTON_MATRIX_KERNEL_CUH
