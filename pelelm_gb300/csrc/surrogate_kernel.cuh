// Fused inference of the learned chemistry surrogate, with the checks that send a cell back to
// the BDF integrator.
//
// The reactor contract is the one of the PelePhysics reactor called by PeleLM::advance_chemistry
// (Source/PeleLM.cpp:5752): advance rhoY, rhoH, T of every unmasked cell over dt_react under
// constant forcing, write FC. Cells the surrogate accepts are written here (FC = 0: no RHS
// evaluation); the others are appended to a device list that the persistent BDF kernel then
// advances in place (ReactParams::cell_list / ncell_dev), with no host round trip.
//
// One CTA of 256 threads owns a tile of 128 consecutive flat cells at a time (persistent over
// tiles):
//   1. featurise (threads 0..127, one cell each): x = [log10 max(Y_k, 1e-14), T, F_k / rho,
//      F_h / rho], z = (x - mean) / std, split into BF16 high and low halves (the first-layer
//      weight is stored twice, so the product carries ~16 bits of z); out-of-range z flags the
//      cell as out of distribution;
//   2. layer stack: the 128-row activation tile stays in shared memory (two ping-pong buffers);
//      weights stream from global/L2 in 32-wide K chunks with cp.async double buffering; 8 warps
//      (4 along cells x 2 along outputs) issue mma.sync m16n8k16 BF16 with FP32 accumulation;
//      bias + GELU epilogue writes the next activation tile as BF16; the output layer writes
//      FP32. Repeated per ensemble member;
//   3. gates and update (threads 0..127, FP64): mean of the ensemble; per-element projection of
//      the predicted chemical source onto exact element conservation (the size of the
//      correction is the conservation check); rhoY_new = rhoY + dt F + rho dY_chem; T from the
//      new (rhoH, Y) by Newton on h(T) (the enthalpy check compares it with the predicted T);
//      negativity, ensemble-disagreement and OOD checks; a hashed 1% sample is routed to the
//      BDF as an audit, its prediction kept for comparison (surrogate_audit_kernel).
#ifndef PGB_SURROGATE_KERNEL_CUH
#define PGB_SURROGATE_KERNEL_CUH

#include <cuda_bf16.h>

#include "mlp_common.cuh"
#include "point_kernels.cuh"
#include "reactor_types.cuh"

namespace pgb {

constexpr int SG_TILE = 128;        // cells per CTA tile
constexpr int SG_WIDTH = 256;       // hidden width
constexpr int SG_MAX_LAYERS = 8;    // hidden layers + output layer
constexpr int SG_MAX_MODELS = 2;    // ensemble members
constexpr int SG_MAX_IN = 128;      // features (2 NS + 2)
constexpr int SG_NOUT_PAD = 32;     // padded outputs
constexpr int SG_MAX_EL = 8;        // elements
constexpr int SG_LDA = SG_WIDTH + 8;  // activation row: 264 bf16 = 528 B (conflict-free ldmatrix)
constexpr int SG_LDW = 32 + 8;        // weight chunk row: 40 bf16 = 80 B
constexpr int SG_LDO = SG_NOUT_PAD + 1;

// Network, normaliser, conservation projection and gate thresholds (device memory, read-only).
struct SurrogateNet {
  int nmodel, nlayer;          // nlayer = hidden layers + 1
  int n_in, k_half, k_in;      // features; split halves start at 0 and k_half; k_in = dims[0]
  int n_out;                   // valid outputs (species with a chemical source, then T)
  int dims[SG_MAX_LAYERS + 1];
  const __nv_bfloat16* W[SG_MAX_MODELS][SG_MAX_LAYERS];  // (dims[l+1] x dims[l]) row-major
  const float* b[SG_MAX_MODELS][SG_MAX_LAYERS];
  float x_mean[SG_MAX_IN], x_inv_std[SG_MAX_IN];
  float z_lo[SG_MAX_IN], z_hi[SG_MAX_IN];   // accepted normalised range (training range + margin)
  double y_scale[SG_NOUT_PAD];
  int out_species[SG_NOUT_PAD];             // species of output j; -1 for T
  int nel;
  double A[SG_MAX_EL][MAXN];                // element e per gram of species k (n_e,k / W_k)
  double P[MAXN][SG_MAX_EL];                // A^T (A A^T)^-1: least-norm restoring correction
  double g_mis, g_cons, g_disT, g_disY, g_neg;  // enthalpy [K], conservation [Y], ensemble [K, Y], Y floor
  double audit_frac, tol_T, tol_Y;
};

struct SurrogateStats {
  unsigned long long ncell, accept, fallback, ood, mis, cons, ens, neg, audit, audit_bad;
  unsigned long long audit_max_dT, audit_max_dY;  // bit patterns of non-negative doubles
};

struct SurrogateParams {
  const BoxDev* boxes;
  int nbox;
  long long ncell;
  double dt;
  const SurrogateNet* net;
  long long* fallback_list;              // capacity ncell
  unsigned long long* fallback_count;
  long long* audit_cell;                 // capacity audit_cap
  double* audit_pred;                    // [audit_cap][MAXN]: predicted Y (NS), then T
  long long audit_cap;
  unsigned long long* audit_count;
  SurrogateStats* stats;
  unsigned long long* seed_dev;          // audit sample seed; advanced by the audit kernel
  float* raw_out;                        // non-null: write the members' raw outputs
                                         // [cell][member][n_out] and leave the state untouched
  float* raw_in;                         // with raw_out: also the network input rows [cell][k_in]
};

__device__ __forceinline__ const BoxDev& sg_locate(const BoxDev* boxes, int nbox, long long c, int& i, int& j,
                                                   int& k, bool& masked) {
  int lo = 0, hi = nbox - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (boxes[mid].cell_offset <= c) lo = mid; else hi = mid - 1;
  }
  const BoxDev& B = boxes[lo];
  long long r = c - B.cell_offset;
  i = B.lo0 + (int)(r % B.len0);
  r /= B.len0;
  j = B.lo1 + (int)(r % B.len1);
  k = B.lo2 + (int)(r / B.len1);
  masked = false;
  if (B.mask.p)
    masked = B.mask.p[(long long)(i - B.mask.begin0) + (long long)(j - B.mask.begin1) * B.mask.jstride +
                      (long long)(k - B.mask.begin2) * B.mask.kstride] < 0;
  return B;
}

__device__ __forceinline__ double sg_uniform(unsigned long long x) {  // splitmix64 finaliser -> [0, 1)
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  x ^= x >> 31;
  return (double)(x >> 11) * (1.0 / 9007199254740992.0);
}

// Raw features of one cell, in FP32, handed to put(q, x): log10 max(Y_k, 1e-14) (q < NS), T,
// F_k / rho (q = NS+1 ..), F_h / rho. The one definition used by the inference kernel and by the
// feature extraction that builds training sets (pgb_surrogate_features), so both see the same bits.
template <class M, class F>
__device__ __forceinline__ void sg_features(const BoxDev& B, int i, int j, int k, F&& put) {
  constexpr int NS = M::NS;
  double rho = 0.0;
#pragma unroll
  for (int s = 0; s < NS; ++s) rho += arr_at(B.rY, i, j, k, s);
  const double inv_rho = 1.0 / rho;
#pragma unroll
  for (int s = 0; s < NS; ++s) put(s, log10f(fmaxf((float)(arr_at(B.rY, i, j, k, s) * inv_rho), 1e-14f)));
  put(NS, (float)arr_at(B.T, i, j, k, 0));
#pragma unroll
  for (int s = 0; s < NS; ++s) put(NS + 1 + s, (float)(arr_at(B.rYsrc, i, j, k, s) * inv_rho));
  put(2 * NS + 1, (float)(arr_at(B.rEsrc, i, j, k, 0) * inv_rho));
}

// One dense layer on the 128-row tile: out = act(in (128 x K) . W^T (K -> N) + b), N = NT * 16.
template <int NT>
__device__ __forceinline__ void sg_layer(const __nv_bfloat16 (*Ain)[SG_LDA], int K, const __nv_bfloat16* __restrict__ W,
                                         const float* __restrict__ bias, __nv_bfloat16 (*Wsm)[SG_WIDTH][SG_LDW],
                                         __nv_bfloat16 (*Aout)[SG_LDA], float (*Oout)[SG_LDO], int n_valid) {
  using namespace pgb_mlp;
  constexpr int N = NT * 16;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = warp >> 1, wn = warp & 1;
  float acc[2][NT][4];
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int r = 0; r < 4; ++r) acc[i][j][r] = 0.f;
  auto load_chunk = [&](int st, int k0) {
    for (int idx = tid; idx < N * 4; idx += 256) {
      const int row = idx >> 2, ch = idx & 3;
      cp_async16(&Wsm[st][row][ch * 8], W + (size_t)row * K + k0 + ch * 8, true);
    }
    cp_async_commit();
  };
  const int nk = K / 32;
  load_chunk(0, 0);
  for (int kt = 0; kt < nk; ++kt) {
    const int st = kt & 1;
    if (kt + 1 < nk) {
      load_chunk(st ^ 1, (kt + 1) * 32);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < 32; kk += 16) {
      unsigned a[2][4], b[NT][2];
#pragma unroll
      for (int i = 0; i < 2; ++i) {
        const int row = wm * 32 + i * 16 + (lane & 15);
        const int col = kt * 32 + kk + (lane >> 4) * 8;
        ldmatrix_x4(a[i][0], a[i][1], a[i][2], a[i][3], &Ain[row][col]);
      }
#pragma unroll
      for (int j = 0; j < NT; j += 2) {
        const int nrow = wn * (NT * 8) + j * 8 + (lane & 7) + ((lane >> 4) << 3);
        const int col = kk + ((lane >> 3) & 1) * 8;
        ldmatrix_x4(b[j][0], b[j][1], b[j + 1][0], b[j + 1][1], &Wsm[st][nrow][col]);
      }
#pragma unroll
      for (int i = 0; i < 2; ++i)
#pragma unroll
        for (int j = 0; j < NT; ++j) mma_bf16(acc[i][j], a[i], b[j]);
    }
    __syncthreads();
  }
#pragma unroll
  for (int i = 0; i < 2; ++i)
#pragma unroll
    for (int j = 0; j < NT; ++j)
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int m = wm * 32 + i * 16 + (lane >> 2) + h * 8;
        const int n = wn * (NT * 8) + j * 8 + (lane & 3) * 2;
#pragma unroll
        for (int e = 0; e < 2; ++e) {
          const float v = acc[i][j][h * 2 + e] + __ldg(bias + n + e);
          if (Aout) Aout[m][n + e] = __float2bfloat16(gelu(v));
          else Oout[m][n + e] = (n + e < n_valid) ? v : 0.f;
        }
      }
  __syncthreads();
}

constexpr size_t sg_smem_bytes() {
  return 2 * sizeof(__nv_bfloat16) * SG_TILE * SG_LDA          // activation ping-pong
         + 2 * sizeof(__nv_bfloat16) * SG_WIDTH * SG_LDW       // weight chunks
         + SG_MAX_MODELS * sizeof(float) * SG_TILE * SG_LDO    // outputs per member
         + sizeof(int) * SG_TILE;                              // OOD flags
}

template <class M>
__global__ void __launch_bounds__(256, 1) surrogate_kernel(const SurrogateParams P) {
  constexpr int NS = M::NS;
  using bf16 = __nv_bfloat16;
  extern __shared__ __align__(16) unsigned char sg_smem[];
  bf16(*A0)[SG_LDA] = reinterpret_cast<bf16(*)[SG_LDA]>(sg_smem);
  bf16(*A1)[SG_LDA] = A0 + SG_TILE;
  bf16(*Wsm)[SG_WIDTH][SG_LDW] = reinterpret_cast<bf16(*)[SG_WIDTH][SG_LDW]>(A1 + SG_TILE);
  float(*O)[SG_TILE][SG_LDO] = reinterpret_cast<float(*)[SG_TILE][SG_LDO]>(Wsm + 2);
  int* ood_flag = reinterpret_cast<int*>(O + SG_MAX_MODELS);
  const SurrogateNet& net = *P.net;
  const int tid = threadIdx.x, lane = tid & 31;
  const unsigned long long seed = *P.seed_dev;

  for (long long tile = blockIdx.x; tile * SG_TILE < P.ncell; tile += gridDim.x) {
    const long long c = tile * SG_TILE + tid;
    for (int mdl = 0; mdl < net.nmodel; ++mdl) {
      // ---- 1. features -> A0 (split BF16), OOD flag
      if (tid < SG_TILE) {
        int ood = 0;
        int i = 0, j = 0, k = 0;
        bool masked = true;
        const BoxDev* B = nullptr;
        if (c < P.ncell) B = &sg_locate(P.boxes, P.nbox, c, i, j, k, masked);
        bf16* row = A0[tid];
        for (int q = 0; q < net.k_in; ++q) row[q] = __float2bfloat16(0.f);
        if (!masked) {
          sg_features<M>(*B, i, j, k, [&](int q, float x) {
            // explicit roundings: a contraction into the last multiply of an inlined log10f
            // would give other bits than the features training saw (pgb_surrogate_features)
            const float z = __fmul_rn(__fsub_rn(x, net.x_mean[q]), net.x_inv_std[q]);
            if (!(z >= net.z_lo[q] && z <= net.z_hi[q])) ood = 1;
            const bf16 hi = __float2bfloat16(z);
            row[q] = hi;
            row[net.k_half + q] = __float2bfloat16(z - __bfloat162float(hi));
          });
        }
        ood_flag[tid] = ood;
      }
      __syncthreads();
      if (P.raw_in && mdl == 0)
        for (int e = tid; e < SG_TILE * net.k_in; e += blockDim.x) {
          const int rr = e / net.k_in, q = e - rr * net.k_in;
          if (tile * SG_TILE + rr < P.ncell) P.raw_in[(size_t)(tile * SG_TILE + rr) * net.k_in + q] = __bfloat162float(A0[rr][q]);
        }
      // ---- 2. layer stack
      bf16(*in)[SG_LDA] = A0;
      bf16(*out)[SG_LDA] = A1;
      for (int l = 0; l + 1 < net.nlayer; ++l) {
        sg_layer<SG_WIDTH / 16>(in, net.dims[l], net.W[mdl][l], net.b[mdl][l], Wsm, out, nullptr, 0);
        bf16(*t)[SG_LDA] = in;
        in = out;
        out = t;
      }
      const int L = net.nlayer - 1;
      sg_layer<SG_NOUT_PAD / 16>(in, net.dims[L], net.W[mdl][L], net.b[mdl][L], Wsm, nullptr, O[mdl], net.n_out);
    }

    if (P.raw_out) {  // raw network outputs only (diagnostics, kernel-vs-training checks)
      if (tid < SG_TILE && c < P.ncell)
        for (int mdl = 0; mdl < net.nmodel; ++mdl)
          for (int q = 0; q < net.n_out; ++q)
            P.raw_out[((size_t)c * net.nmodel + mdl) * net.n_out + q] = O[mdl][tid][q];
      __syncthreads();
      continue;
    }
    // ---- 3. gates and update (warps 0..3: whole warps, so the ballots below are full)
    if (tid < SG_TILE) {
      SurrogateStats* S = P.stats;
      int i = 0, j = 0, k = 0;
      bool masked = true;
      const BoxDev* B = nullptr;
      if (c < P.ncell) B = &sg_locate(P.boxes, P.nbox, c, i, j, k, masked);
      bool active = !masked;
      bool f_ood = false, f_mis = false, f_cons = false, f_ens = false, f_neg = false;
      bool accept = false, audit = false;
      double rY1[NS], Y1[NS], Th = 0.0, rE1 = 0.0;
      if (active) {
        double dY[NS], rho0 = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) { dY[s] = 0.0; rho0 += arr_at(B->rY, i, j, k, s); }
        const int nm = net.nmodel;
        double dT = 0.0, disT = 0.0, disY = 0.0;
        for (int q = 0; q < net.n_out; ++q) {
          const double o0 = O[0][tid][q];
          const double o1 = (nm > 1) ? (double)O[1][tid][q] : o0;
          const double v = 0.5 * (o0 + o1) * net.y_scale[q];
          const double d = fabs(o0 - o1) * net.y_scale[q];
          const int s = net.out_species[q];
          if (s < 0) { dT = v; disT = d; }
          else {
#pragma unroll
            for (int u = 0; u < NS; ++u) if (u == s) dY[u] = v;
            disY = fmax(disY, d);
          }
        }
        // element conservation: least-norm correction restoring sum_k A_ek dY_k = 0
        double viol[SG_MAX_EL];
        for (int e = 0; e < net.nel; ++e) {
          double a = 0.0;
#pragma unroll
          for (int s = 0; s < NS; ++s) a = fma(net.A[e][s], dY[s], a);
          viol[e] = a;
        }
        double cons = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          double corr = 0.0;
          for (int e = 0; e < net.nel; ++e) corr = fma(-net.P[s][e], viol[e], corr);
          dY[s] += corr;
          cons = fmax(cons, fabs(corr));
        }
        double rho1 = 0.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) {
          rY1[s] = fma(P.dt, arr_at(B->rYsrc, i, j, k, s), arr_at(B->rY, i, j, k, s)) + rho0 * dY[s];
          rho1 += rY1[s];
        }
        const double inv_rho1 = 1.0 / rho1;
        double ymin = 1.0;
#pragma unroll
        for (int s = 0; s < NS; ++s) { Y1[s] = rY1[s] * inv_rho1; ymin = fmin(ymin, Y1[s]); }
        rE1 = fma(P.dt, arr_at(B->rEsrc, i, j, k, 0), arr_at(B->rE, i, j, k, 0));
        const double Tp = arr_at(B->T, i, j, k, 0) + dT;
        Th = hy2t_newton<M>(rE1 * inv_rho1, Y1, Tp, 90.0, 5000.0);
        f_ood = ood_flag[tid] != 0;
        f_mis = !(fabs(Th - Tp) <= net.g_mis) || !(Th > 90.0 && Th < 5000.0);
        f_cons = !(cons <= net.g_cons);
        f_ens = !(disT <= net.g_disT && disY <= net.g_disY);
        f_neg = !(ymin >= -net.g_neg) || !(rho1 > 0.0);
        accept = !(f_ood || f_mis || f_cons || f_ens || f_neg);
        if (accept && net.audit_frac > 0.0 && sg_uniform((unsigned long long)c ^ seed) < net.audit_frac) {
          const unsigned long long a = atomicAdd(P.audit_count, 1ull);
          if ((long long)a < P.audit_cap) {
            audit = true;
            P.audit_cell[a] = c;
            double* pr = P.audit_pred + (size_t)a * MAXN;
#pragma unroll
            for (int s = 0; s < NS; ++s) pr[s] = Y1[s];
            pr[NS] = Th;
          }
        }
        if (accept && !audit) {
#pragma unroll
          for (int s = 0; s < NS; ++s) arr_at(B->rY, i, j, k, s) = rY1[s];
          arr_at(B->rE, i, j, k, 0) = rE1;
          arr_at(B->T, i, j, k, 0) = Th;
          arr_at(B->FC, i, j, k, 0) = 0.0;
        }
      } else if (B) {
        arr_at(B->FC, i, j, k, 0) = 0.0;  // covered cell
      }
      const bool to_bdf = active && !(accept && !audit);
      const unsigned fb = __ballot_sync(0xffffffffu, to_bdf);
      if (fb) {
        const int leader = __ffs(fb) - 1;
        unsigned long long base = 0;
        if (lane == leader) base = atomicAdd(P.fallback_count, (unsigned long long)__popc(fb));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (to_bdf) P.fallback_list[base + __popc(fb & ((1u << lane) - 1u))] = c;
      }
      const unsigned n_act = __popc(__ballot_sync(0xffffffffu, active));
      const unsigned n_acc = __popc(__ballot_sync(0xffffffffu, accept && !audit));
      const unsigned n_ood = __popc(__ballot_sync(0xffffffffu, f_ood));
      const unsigned n_mis = __popc(__ballot_sync(0xffffffffu, f_mis));
      const unsigned n_cons = __popc(__ballot_sync(0xffffffffu, f_cons));
      const unsigned n_ens = __popc(__ballot_sync(0xffffffffu, f_ens));
      const unsigned n_neg = __popc(__ballot_sync(0xffffffffu, f_neg));
      const unsigned n_aud = __popc(__ballot_sync(0xffffffffu, audit));
      if (lane == 0) {
        if (n_act) atomicAdd(&S->ncell, (unsigned long long)n_act);
        if (n_acc) atomicAdd(&S->accept, (unsigned long long)n_acc);
        if (__popc(fb)) atomicAdd(&S->fallback, (unsigned long long)__popc(fb));
        if (n_ood) atomicAdd(&S->ood, (unsigned long long)n_ood);
        if (n_mis) atomicAdd(&S->mis, (unsigned long long)n_mis);
        if (n_cons) atomicAdd(&S->cons, (unsigned long long)n_cons);
        if (n_ens) atomicAdd(&S->ens, (unsigned long long)n_ens);
        if (n_neg) atomicAdd(&S->neg, (unsigned long long)n_neg);
        if (n_aud) atomicAdd(&S->audit, (unsigned long long)n_aud);
      }
    }
    __syncthreads();
  }
}

// Raw features of every cell (flat cell order) into out[c * (2 NS + 2) + q]; masked cells get 0.
template <class M>
__global__ void surrogate_features_kernel(const BoxDev* boxes, int nbox, long long ncell, float* out) {
  constexpr int NIN = 2 * M::NS + 2;
  for (long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x; c < ncell; c += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    bool masked;
    const BoxDev& B = sg_locate(boxes, nbox, c, i, j, k, masked);
    float* o = out + c * NIN;
    if (masked) {
      for (int q = 0; q < NIN; ++q) o[q] = 0.f;
    } else {
      sg_features<M>(B, i, j, k, [&](int q, float x) { __stcg(o + q, x); });
    }
  }
}

// After the BDF has advanced the fallback cells: compares each audited cell's BDF result with
// the surrogate's prediction kept for it.
template <class M>
__global__ void surrogate_audit_kernel(const SurrogateParams P) {
  constexpr int NS = M::NS;
  const SurrogateNet& net = *P.net;
  const long long n = min((long long)*P.audit_count, P.audit_cap);
  if (blockIdx.x == 0 && threadIdx.x == 0) *P.seed_dev += 0x9E3779B97F4A7C15ull;  // next call's sample
  for (long long a = (long long)blockIdx.x * blockDim.x + threadIdx.x; a < n; a += (long long)gridDim.x * blockDim.x) {
    int i, j, k;
    bool masked;
    const BoxDev& B = sg_locate(P.boxes, P.nbox, P.audit_cell[a], i, j, k, masked);
    const double* pr = P.audit_pred + (size_t)a * MAXN;
    double rho = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s) rho += arr_at(B.rY, i, j, k, s);
    double eY = 0.0;
#pragma unroll
    for (int s = 0; s < NS; ++s) eY = fmax(eY, fabs(arr_at(B.rY, i, j, k, s) / rho - pr[s]));
    const double eT = fabs(arr_at(B.T, i, j, k, 0) - pr[NS]);
    atomicMax(&P.stats->audit_max_dT, (unsigned long long)__double_as_longlong(eT));
    atomicMax(&P.stats->audit_max_dY, (unsigned long long)__double_as_longlong(eY));
    if (!(eT <= net.tol_T && eY <= net.tol_Y)) atomicAdd(&P.stats->audit_bad, 1ull);
  }
}

}  // namespace pgb

#endif  // PGB_SURROGATE_KERNEL_CUH
