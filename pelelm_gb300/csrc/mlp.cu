// BF16 tensor-core kernels of the learned chemistry surrogate: GEMM with fused epilogues,
// transposes, GELU backward, loss gradient, bias gradients and Adam. FP32 accumulation and FP32
// master weights throughout; BF16 operands.
//
// GEMM convention ("NT"): C[m][n] = sum_k A[m][k] * B[n][k], A (M x K) and B (N x K) row-major
// with K contiguous. Forward layers store W as (out x in); the backward products use explicit
// transposes so every product is this one tiled kernel.
//
// Tiling: 128 x 128 CTA tile, 32-wide K steps double-buffered with cp.async, 8 warps in a 4 x 2
// grid, each warp a 32 x 64 tile of mma.sync.m16n8k16 (bf16 in, fp32 accumulate) fed by
// ldmatrix from padded shared rows (no bank conflicts). Shapes are padded by the host so M, N
// are multiples of 16 and K a multiple of 32.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "reactor_registry.cuh"

#include "mlp_common.cuh"

namespace pgb_mlp {

constexpr int BM = 128, BN = 128, BK = 32, PAD = 8, LDS = BK + PAD;  // shared row: 40 bf16 = 80 B

// Epilogue arguments: out = act(acc + bias); optional FP32 pre-activation, BF16 and/or FP32 out.
struct Epi {
  const float* bias;  // [N] or null
  int act;            // 0 identity, 1 GELU
  float* pre;         // [M][ldo] FP32 pre-activation, or null
  bf16* out_bf16;     // [M][ldo], or null
  float* out_f32;     // [M][ldo], or null
  int ldo;
  int n_valid;        // columns >= n_valid are written as 0 (padding)
};

__global__ void __launch_bounds__(256) gemm_nt_kernel(const bf16* __restrict__ A, int lda,
                                                      const bf16* __restrict__ B, int ldb, int M, int N,
                                                      int K, Epi epi) {
  __shared__ __align__(16) bf16 As[2][BM][LDS];
  __shared__ __align__(16) bf16 Bs[2][BN][LDS];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;  // 4 x 2 warps: 32 x 64 each
  const int m0 = blockIdx.y * BM, n0 = blockIdx.x * BN;
  float acc[2][8][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;

  auto load_stage = [&](int st, int k0) {
#pragma unroll
    for (int c = 0; c < 2; ++c) {  // 128 rows x 4 chunks of 8 bf16 = 512 chunks per operand
      const int idx = tid + c * 256;
      const int row = idx >> 2, ch = idx & 3;
      const int gm = m0 + row, gn = n0 + row, gk = k0 + ch * 8;
      cp_async16(&As[st][row][ch * 8], A + (size_t)min(gm, M - 1) * lda + gk, gm < M);
      cp_async16(&Bs[st][row][ch * 8], B + (size_t)min(gn, N - 1) * ldb + gk, gn < N);
    }
    cp_async_commit();
  };

  const int nk = K / BK;
  load_stage(0, 0);
  for (int kt = 0; kt < nk; ++kt) {
    const int st = kt & 1;
    if (kt + 1 < nk) {
      load_stage(st ^ 1, (kt + 1) * BK);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < BK; kk += 16) {
      unsigned a[2][4], b[8][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int row = wm * 32 + i * 16 + (lane & 15);
        const int col = kk + (lane >> 4) * 8;
        ldmatrix_x4(a[i][0], a[i][1], a[i][2], a[i][3], &As[st][row][col]);
      }
#pragma unroll
      for (int j = 0; j < 8; j += 2) {  // two n8 tiles per ldmatrix.x4
        const int nrow = wn * 64 + j * 8 + (lane & 7) + ((lane >> 4) << 3);
        const int col = kk + ((lane >> 3) & 1) * 8;
        ldmatrix_x4(b[j][0], b[j][1], b[j + 1][0], b[j + 1][1], &Bs[st][nrow][col]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) mma_bf16(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
  // epilogue
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < 8; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int m = m0 + wm * 32 + i * 16 + (lane >> 2) + h * 8;
        const int n = n0 + wn * 64 + j * 8 + (lane & 3) * 2;
        if (m >= M) continue;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const int nn = n + e;
          if (nn >= N) continue;
          float v = acc[i][j][h * 2 + e];
          if (epi.bias) v += epi.bias[nn];
          if (epi.pre) epi.pre[(size_t)m * epi.ldo + nn] = v;
          if (epi.act == 1) v = gelu(v);
          if (nn >= epi.n_valid) v = 0.f;
          if (epi.out_bf16) epi.out_bf16[(size_t)m * epi.ldo + nn] = __float2bfloat16(v);
          if (epi.out_f32) epi.out_f32[(size_t)m * epi.ldo + nn] = v;
        }
      }
}

// out[c][r] = in[r][c] (rows x cols -> cols x rows), bf16, 32 x 32 tiles through shared memory.
__global__ void transpose_bf16_kernel(const bf16* __restrict__ in, int rows, int cols, int ldi,
                                      bf16* __restrict__ out, int ldo) {
  __shared__ bf16 t[32][33];
  const int c0 = blockIdx.x * 32, r0 = blockIdx.y * 32;
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int r = r0 + y, c = c0 + threadIdx.x;
    t[y][threadIdx.x] = (r < rows && c < cols) ? in[(size_t)r * ldi + c] : __float2bfloat16(0.f);
  }
  __syncthreads();
  for (int y = threadIdx.y; y < 32; y += 8) {
    const int c = c0 + y, r = r0 + threadIdx.x;
    if (c < cols && r < rows) out[(size_t)c * ldo + r] = t[threadIdx.x][y];
  }
}

// dZ = dA * gelu'(pre) (FP32 in, BF16 out), elementwise over n elements.
__global__ void gelu_backward_kernel(const float* __restrict__ dA, const float* __restrict__ pre,
                                     bf16* __restrict__ dZ, float* __restrict__ dZf, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float g = dA[i] * gelu_grad(pre[i]);
    dZ[i] = __float2bfloat16(g);
    if (dZf) dZf[i] = g;
  }
}

// Mean-squared-error gradient on the first n_valid of ld columns: dY = 2 (Y - T) / (M n_valid);
// also accumulates the loss sum into *loss.
__global__ void mse_grad_kernel(const float* __restrict__ Y, const float* __restrict__ T, int M, int ld,
                                int n_valid, float* __restrict__ dYf, bf16* __restrict__ dY,
                                float* __restrict__ loss) {
  float local = 0.f;
  const float scale = 2.f / ((float)M * (float)n_valid);
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < (long long)M * ld;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % ld);
    float g = 0.f;
    if (c < n_valid) {
      const float d = Y[i] - T[i];
      local += d * d;
      g = scale * d;
    }
    dYf[i] = g;
    dY[i] = __float2bfloat16(g);
  }
  for (int o = 16; o; o >>= 1) local += __shfl_xor_sync(0xffffffffu, local, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, local);
}

// db[n] = sum_m dZ[m][n] (FP32), one block per 32 columns.
__global__ void bias_grad_kernel(const float* __restrict__ dZ, int M, int N, int ld, float* __restrict__ db) {
  __shared__ float s[8][33];
  const int n = blockIdx.x * 32 + threadIdx.x;
  float acc = 0.f;
  if (n < N)
    for (int m = threadIdx.y; m < M; m += 8) acc += dZ[(size_t)m * ld + n];
  s[threadIdx.y][threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.y == 0 && n < N) {
    float t = 0.f;
    for (int y = 0; y < 8; ++y) t += s[y][threadIdx.x];
    db[n] = t;
  }
}

// Adam on FP32 master parameters; refreshes the BF16 copy used by the GEMMs.
__global__ void adam_kernel(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                            float* __restrict__ v, bf16* __restrict__ p_bf16, long long n, float lr,
                            float b1, float b2, float eps, float bc1, float bc2) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float pi = p[i] - lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
    p[i] = pi;
    if (p_bf16) p_bf16[i] = __float2bfloat16(pi);
  }
}

__global__ void f32_to_bf16_kernel(const float* __restrict__ in, bf16* __restrict__ out, long long n) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    out[i] = __float2bfloat16(in[i]);
}

// Row r of W (rows x cols, FP32) -> BF16 twice, at out[r*ldo + c] and out[r*ldo + cols + c]: the
// first-layer weight seen by an input split into high and low BF16 halves (split_rows_kernel).
__global__ void dup_weight_kernel(const float* __restrict__ W, int rows, int cols, bf16* __restrict__ out,
                                  int ldo) {
  const long long n = (long long)rows * cols;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const bf16 w = __float2bfloat16(W[i]);
    out[(long long)r * ldo + c] = w;
    out[(long long)r * ldo + cols + c] = w;
  }
}

// x (FP32) -> hi = bf16(x) at column c, lo = bf16(x - hi) at column off + c: with FP32 accumulation
// the pair carries ~16 significant bits of x through a BF16 GEMM.
__global__ void split_rows_kernel(const float* __restrict__ x, int rows, int cols, int ldx, bf16* __restrict__ out,
                                  int ldo, int off) {
  const long long n = (long long)rows * cols;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const int r = (int)(i / cols), c = (int)(i % cols);
    const float v = x[(long long)r * ldx + c];
    const bf16 hi = __float2bfloat16(v);
    out[(long long)r * ldo + c] = hi;
    out[(long long)r * ldo + off + c] = __float2bfloat16(v - __bfloat162float(hi));
  }
}

}  // namespace pgb_mlp

using namespace pgb_host;
using pgb_mlp::bf16;

static int grid_for(long long n) { return (int)std::min<long long>((n + 255) / 256, 4096); }

extern "C" {

int pgb_mlp_gemm_nt(const void* A, int lda, const void* B, int ldb, int M, int N, int K,
                    const float* bias, int act, float* pre, void* out_bf16, float* out_f32, int ldo,
                    int n_valid, void* stream) {
  if (M <= 0 || N <= 0 || K <= 0 || K % 32 || lda % 8 || ldb % 8)
    return set_err("gemm_nt: need M,N,K > 0, K %% 32 == 0, lda/ldb multiples of 8");
  pgb_mlp::Epi e{bias, act, pre, static_cast<bf16*>(out_bf16), out_f32, ldo, n_valid};
  dim3 grid((N + pgb_mlp::BN - 1) / pgb_mlp::BN, (M + pgb_mlp::BM - 1) / pgb_mlp::BM);
  pgb_mlp::gemm_nt_kernel<<<grid, 256, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(A), lda, static_cast<const bf16*>(B), ldb, M, N, K, e);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

int pgb_mlp_transpose_bf16(const void* in, int rows, int cols, int ldi, void* out, int ldo, void* stream) {
  dim3 grid((cols + 31) / 32, (rows + 31) / 32), block(32, 8);
  pgb_mlp::transpose_bf16_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(
      static_cast<const bf16*>(in), rows, cols, ldi, static_cast<bf16*>(out), ldo);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

int pgb_mlp_gelu_backward(const float* dA, const float* pre, void* dZ, float* dZf, long long n, void* stream) {
  pgb_mlp::gelu_backward_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      dA, pre, static_cast<bf16*>(dZ), dZf, n);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

int pgb_mlp_mse_grad(const float* Y, const float* T, int M, int ld, int n_valid, float* dYf, void* dY,
                     float* loss, void* stream) {
  pgb_mlp::mse_grad_kernel<<<grid_for((long long)M * ld), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      Y, T, M, ld, n_valid, dYf, static_cast<bf16*>(dY), loss);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

int pgb_mlp_bias_grad(const float* dZ, int M, int N, int ld, float* db, void* stream) {
  dim3 grid((N + 31) / 32), block(32, 8);
  pgb_mlp::bias_grad_kernel<<<grid, block, 0, static_cast<cudaStream_t>(stream)>>>(dZ, M, N, ld, db);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

int pgb_mlp_adam(float* p, const float* g, float* m, float* v, void* p_bf16, long long n, float lr,
                 float b1, float b2, float eps, int step, void* stream) {
  if (step < 1) return set_err("adam: step must be >= 1");
  const float bc1 = 1.f - powf(b1, (float)step), bc2 = 1.f - powf(b2, (float)step);
  pgb_mlp::adam_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      p, g, m, v, static_cast<bf16*>(p_bf16), n, lr, b1, b2, eps, bc1, bc2);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

int pgb_mlp_f32_to_bf16(const float* in, void* out, long long n, void* stream) {
  pgb_mlp::f32_to_bf16_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      in, static_cast<bf16*>(out), n);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

int pgb_mlp_dup_weight_bf16(const float* W, int rows, int cols, void* out, int ldo, void* stream) {
  if (rows <= 0 || cols <= 0 || ldo < 2 * cols) return set_err("dup_weight: need ldo >= 2*cols");
  pgb_mlp::dup_weight_kernel<<<grid_for((long long)rows * cols), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      W, rows, cols, static_cast<bf16*>(out), ldo);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

int pgb_mlp_split_rows_bf16(const float* x, int rows, int cols, int ldx, void* out, int ldo, int off,
                            void* stream) {
  if (rows <= 0 || cols <= 0 || off < cols || ldo < off + cols || ldx < cols)
    return set_err("split_rows: need cols <= off and off + cols <= ldo");
  pgb_mlp::split_rows_kernel<<<grid_for((long long)rows * cols), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      x, rows, cols, ldx, static_cast<bf16*>(out), ldo, off);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

}  // extern "C"
