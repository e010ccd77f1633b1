// Mechanism registry shared by the per-mechanism translation units and the host driver.
// Each mech_<name>.cu instantiates the kernels of one mechanism and exports one MechEntry.
#ifndef PGB_REACTOR_REGISTRY_CUH
#define PGB_REACTOR_REGISTRY_CUH

#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "../../include/pelelm_gb300.h"
#include "bdf_group_kernel.cuh"
#include "newton_matrix_kernel.cuh"
#include "bdf_kernel.cuh"
#include "bdf_warp_kernel.cuh"
#include "point_kernels.cuh"
#include "reactor_types.cuh"
#include "surrogate_kernel.cuh"

namespace pgb_host {

// Records the calling thread's error message (pgb_last_error) and returns -1.
int set_err(const char* fmt, ...);

#define PGB_CUDA(call)                                                                       \
  do {                                                                                       \
    cudaError_t e_ = (call);                                                                 \
    if (e_ != cudaSuccess) return ::pgb_host::set_err("%s: %s (%s:%d)", #call,              \
                                                      cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

using LaunchFn = int (*)(const pgb::ReactParams&, int tpb, cudaStream_t, int nblocks);

constexpr int kMaxSmemPerBlock = 227 * 1024;

template <class M, class JR, int TPB, int LAYOUT>
int launch_bdf_tpb(const pgb::ReactParams& p, cudaStream_t s, int nblocks) {
  constexpr int smem = pgb::bdf_smem_per_thread<M, JR, LAYOUT>() * TPB;
  if constexpr (smem > kMaxSmemPerBlock) {
    return set_err("%s: %d threads per block need %d B of shared memory (limit %d)", M::NAME, TPB,
                   smem, kMaxSmemPerBlock);
  } else {
    auto kern = pgb::bdf_reactor_kernel<M, JR, TPB, LAYOUT>;
    PGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    kern<<<nblocks, TPB, smem, s>>>(p);
    PGB_CUDA(cudaGetLastError());
    return 0;
  }
}

template <class M, class JR, int LAYOUT>
int launch_bdf_layout(const pgb::ReactParams& p, int tpb, cudaStream_t s, int nblocks) {
  // 64 threads only for the all-shared layout (the allocation-free entry's fallback), 256 only
  // for the global layouts
  if (tpb == 128) return launch_bdf_tpb<M, JR, 128, LAYOUT>(p, s, nblocks);
  if constexpr (LAYOUT == 0) {
    if (tpb == 64) return launch_bdf_tpb<M, JR, 64, LAYOUT>(p, s, nblocks);
  } else {
    if (tpb == 256) return launch_bdf_tpb<M, JR, 256, LAYOUT>(p, s, nblocks);
  }
  return set_err("gb.tpb=%d is not compiled for this layout (64/128 shared, 128/256 global)", tpb);
}

// Launches the persistent BDF kernel with `tpb` threads per block; the Jacobian/LU slices and
// the Nordsieck histories go to p.lu_scratch / p.z_scratch when those are set (sized for
// nblocks * tpb threads), else to shared memory.
template <class M, class JR>
int launch_bdf(const pgb::ReactParams& p, int tpb, cudaStream_t s, int nblocks) {
  const int layout = (p.lu_scratch ? pgb::LAYOUT_LU_GLOBAL : 0) | (p.z_scratch ? pgb::LAYOUT_Z_GLOBAL : 0);
  switch (layout) {
    case 0: return launch_bdf_layout<M, JR, 0>(p, tpb, s, nblocks);
    case 2: return launch_bdf_layout<M, JR, 2>(p, tpb, s, nblocks);
    case 3: return launch_bdf_layout<M, JR, 3>(p, tpb, s, nblocks);
    default: return set_err("a global Jacobian/LU without a global history is not compiled");
  }
}

// Warp-per-cell BDF: `wpb` warps per block, one persistent block per SM.
template <class M, class JR, int WPB>
int launch_bdf_warp_wpb(const pgb::ReactParams& p, cudaStream_t s, int nblocks) {
  constexpr int smem = WPB * pgb::bdf_warp_smem_per_warp<M, JR>();
  if constexpr (smem > kMaxSmemPerBlock) {
    return set_err("warp BDF: %d warps x %d B shared memory exceed the %d B per block", WPB,
                   pgb::bdf_warp_smem_per_warp<M, JR>(), kMaxSmemPerBlock);
  } else {
    auto kern = pgb::bdf_warp_kernel<M, JR, WPB>;
    PGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    kern<<<nblocks, WPB * 32, smem, s>>>(p);
    PGB_CUDA(cudaGetLastError());
    return 0;
  }
}

// Warps per block compiled for a mechanism, most preferred first (0 ends the list): one size
// for small mechanisms (the warp mapping is not their default), 16 for mid-sized ones (more
// resident warps hide the latency of the lane-parallel RHS; 24 measured slower: the register
// cap then spills), what shared memory allows for the large ones.
template <class M>
constexpr int warp_wpb_choice(int i) {
  if constexpr (M::NS <= 12) {
    return i == 0 ? 8 : 0;
  } else if constexpr (M::N <= 32) {
    constexpr int c[] = {16, 8, 0, 0};
    return i < 4 ? c[i] : 0;
  } else {
    constexpr int c[] = {8, 6, 4, 0};
    return i < 4 ? c[i] : 0;
  }
}

template <class M, class JR>
int launch_bdf_warp(const pgb::ReactParams& p, int wpb, cudaStream_t s, int nblocks) {
  if constexpr (M::NS <= 12) {
    if (wpb == 8) return launch_bdf_warp_wpb<M, JR, 8>(p, s, nblocks);
  } else if constexpr (M::N <= 32) {
    if (wpb == 16) return launch_bdf_warp_wpb<M, JR, 16>(p, s, nblocks);
    if (wpb == 8) return launch_bdf_warp_wpb<M, JR, 8>(p, s, nblocks);
  } else {
    if (wpb == 8) return launch_bdf_warp_wpb<M, JR, 8>(p, s, nblocks);
    if (wpb == 6) return launch_bdf_warp_wpb<M, JR, 6>(p, s, nblocks);
    if (wpb == 4) return launch_bdf_warp_wpb<M, JR, 4>(p, s, nblocks);
  }
  return set_err("warp BDF: %d warps per block are not compiled for %s", wpb, M::NAME);
}

// Group-per-cell BDF: G lanes per cell, as many warps per block as fit shared memory (at most
// 16), one persistent block per SM.
template <class M, class JR, int G>
constexpr int group_wpb() {
  constexpr int per = pgb::gbdf_smem_per_warp<M, JR, G>();
  constexpr int w = kMaxSmemPerBlock / per;
  return w > 16 ? 16 : w;
}

template <class M, class JR, int G>
int launch_bdf_group_g(const pgb::ReactParams& p, cudaStream_t s, int nblocks) {
  constexpr int WPB = group_wpb<M, JR, G>();
  if constexpr (WPB < 1) {
    return set_err("group BDF: one warp of %d-lane groups needs %d B of shared memory (limit %d)", G,
                   pgb::gbdf_smem_per_warp<M, JR, G>(), kMaxSmemPerBlock);
  } else {
    constexpr int smem = WPB * pgb::gbdf_smem_per_warp<M, JR, G>();
    auto kern = pgb::bdf_group_kernel<M, JR, G, WPB>;
    PGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    kern<<<nblocks, WPB * 32, smem, s>>>(p);
    PGB_CUDA(cudaGetLastError());
    return 0;
  }
}

// Cells one block of the group kernel holds (warps per block x cells per warp).
template <class M, class JR>
int group_cells_per_block(int G) {
  if (G == 8) return group_wpb<M, JR, 8>() * 4;
  if (G == 4) return group_wpb<M, JR, 4>() * 8;
  return 0;
}

// The group size is the launch argument (LaunchFn's second parameter).
template <class M, class JR>
int launch_bdf_group(const pgb::ReactParams& p, int G, cudaStream_t s, int nblocks) {
  if (G == 8) return launch_bdf_group_g<M, JR, 8>(p, s, nblocks);
  if (G == 4) return launch_bdf_group_g<M, JR, 4>(p, s, nblocks);
  return set_err("group BDF: %d lanes per cell are not compiled (4, 8)", G);
}

template <class M>
int launch_null(const pgb::ReactParams& p, cudaStream_t s, int nblocks) {
  pgb::null_reactor_kernel<M><<<nblocks, 256, 0, s>>>(p);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

template <class M>
int launch_surrogate(const pgb::SurrogateParams& p, cudaStream_t s, int nblocks) {
  constexpr int smem = (int)pgb::sg_smem_bytes();
  static_assert(smem <= kMaxSmemPerBlock, "surrogate tile does not fit shared memory");
  auto kern = pgb::surrogate_kernel<M>;
  PGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
  kern<<<nblocks, 256, smem, s>>>(p);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

template <class M>
int launch_surrogate_audit(const pgb::SurrogateParams& p, cudaStream_t s, int nblocks) {
  pgb::surrogate_audit_kernel<M><<<nblocks, 256, 0, s>>>(p);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

template <class M>
int launch_surrogate_features(const pgb::BoxDev* boxes, int nbox, long long ncell, float* out, cudaStream_t s) {
  const long long nb = std::min<long long>((ncell + 255) / 256, 4096);
  pgb::surrogate_features_kernel<M><<<(int)std::max<long long>(nb, 1), 256, 0, s>>>(boxes, nbox, ncell, out);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

struct MechEntry {
  const char* name;
  int ns, nr;
  LaunchFn bdf_mixed, bdf_fp64;
  int (*null_fn)(const pgb::ReactParams&, cudaStream_t, int);
  int smem_mixed, smem_fp64;  // shared bytes per thread, everything in shared memory
  int smem_mixed_g, smem_fp64_g;  // shared bytes per thread, Nordsieck history in global scratch
  int smem_mixed_gl, smem_fp64_gl;  // shared bytes per thread, history and LU in global scratch
  int (*rates_fn)(const pgb_box_view*, const pgb_array4*, cudaStream_t);
  int (*h2t_fn)(const pgb_box_view*, double, double, cudaStream_t);
  int (*sg_fn)(const pgb::SurrogateParams&, cudaStream_t, int);
  int (*sg_audit_fn)(const pgb::SurrogateParams&, cudaStream_t, int);
  LaunchFn warp_mixed, warp_fp64;  // warp-per-cell BDF (argument: warps per block)
  int wsmem_mixed, wsmem_fp64;     // shared bytes per warp
  int (*sg_feat_fn)(const pgb::BoxDev*, int, long long, float*, cudaStream_t);
  int wpb_choice[4];  // warps per block compiled for the warp kernel, preferred first, 0-ended
  int (*hr_fn)(const pgb_box*, const pgb_array4*, const pgb_array4*, const pgb_array4*, cudaStream_t);
  LaunchFn group_mixed, group_fp64;  // group-per-cell BDF (argument: lanes per cell, 4 or 8)
  int (*group_cells_mixed)(int), (*group_cells_fp64)(int);  // cells per block for a group size
  int (*newton_fn)(const pgb::NewtonMatrixParams&, int mapping, int fp64, cudaStream_t);  // diagnostic
};



inline pgb::ArrDev arr_dev(const pgb_array4& a) {
  pgb::ArrDev d;
  d.p = static_cast<double*>(a.p);
  d.jstride = a.jstride;
  d.kstride = a.kstride;
  d.nstride = a.nstride;
  d.begin0 = a.begin[0];
  d.begin1 = a.begin[1];
  d.begin2 = a.begin[2];
  return d;
}

inline int check_arr(const pgb_array4& a, const pgb_box& b, int ncomp, const char* what, int ibox) {
  if (!a.p) return set_err("box %d: array %s is NULL", ibox, what);
  for (int d = 0; d < 3; ++d)
    if (b.lo[d] < a.begin[d] || b.hi[d] >= a.end[d])
      return set_err("box %d: array %s [%d,%d) in dim %d does not cover the box [%d,%d]", ibox,
                     what, a.begin[d], a.end[d], d, b.lo[d], b.hi[d]);
  if (a.ncomp < ncomp) return set_err("box %d: array %s has %d comps, need %d", ibox, what, a.ncomp, ncomp);
  return 0;
}

template <class M>
int rates_entry(const pgb_box_view* v, const pgb_array4* out, cudaStream_t s) {
  const pgb_box& b = v->box;
  if (check_arr(v->rY, b, M::NS, "rY", 0) || check_arr(v->T, b, 1, "T", 0) ||
      check_arr(v->rEner, b, 1, "rEner", 0) || check_arr(*out, b, M::NS, "out", 0))
    return -1;
  if (v->mask.p && check_arr(v->mask, b, 1, "mask", 0)) return -1;
  pgb::PointParams p;
  p.lo0 = b.lo[0]; p.lo1 = b.lo[1]; p.lo2 = b.lo[2];
  p.len0 = b.hi[0] - b.lo[0] + 1; p.len1 = b.hi[1] - b.lo[1] + 1; p.len2 = b.hi[2] - b.lo[2] + 1;
  p.rY = arr_dev(v->rY); p.rE = arr_dev(v->rEner); p.T = arr_dev(v->T); p.out = arr_dev(*out);
  p.mask.p = static_cast<const int*>(v->mask.p);
  p.mask.jstride = v->mask.jstride; p.mask.kstride = v->mask.kstride;
  p.mask.begin0 = v->mask.begin[0]; p.mask.begin1 = v->mask.begin[1]; p.mask.begin2 = v->mask.begin[2];
  const long long n = (long long)p.len0 * p.len1 * p.len2;
  if (n == 0) return 0;
  pgb::rates_kernel<M><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(p);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

// Newton matrix pieces of the warp / lane-group setup for a batch of states (diagnostic).
template <class M, class JR>
int launch_newton_matrix_jr(const pgb::NewtonMatrixParams& p, cudaStream_t s, int nsm) {
  constexpr int smem = pgb::newton_matrix_smem<M, JR>();
  if constexpr (smem > kMaxSmemPerBlock) {
    return set_err("newton matrix: %d B of shared memory per cell exceed %d B", smem, kMaxSmemPerBlock);
  } else {
    auto kern = pgb::newton_matrix_kernel<M, JR>;
    PGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const long long nb = std::min<long long>(p.ncell, (long long)nsm * 8);
    kern<<<(unsigned)nb, 32, smem, s>>>(p);
    PGB_CUDA(cudaGetLastError());
    return 0;
  }
}
template <class M, class JR>
int launch_newton_matrix_thread_jr(const pgb::NewtonMatrixParams& p, cudaStream_t s, int nsm) {
  constexpr int smem = pgb::newton_matrix_thread_smem<M, JR>();
  if constexpr (smem > kMaxSmemPerBlock) {
    return set_err("newton matrix: %d B of shared memory per block exceed %d B", smem, kMaxSmemPerBlock);
  } else {
    auto kern = pgb::newton_matrix_thread_kernel<M, JR>;
    PGB_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, smem));
    const long long nb = std::min<long long>((p.ncell + 31) / 32, (long long)nsm * 8);
    kern<<<(unsigned)nb, 32, smem, s>>>(p);
    PGB_CUDA(cudaGetLastError());
    return 0;
  }
}
// mapping 1: warp / lane-group kernels; mapping 0: cell-per-thread kernels (THREAD: compiled)
template <class M, bool THREAD>
int newton_matrix_entry(const pgb::NewtonMatrixParams& p, int mapping, int fp64, cudaStream_t s) {
  if (mapping != 0 && mapping != 1) return set_err("newton matrix: mapping must be 0 (per thread) or 1 (per warp)");
  if (p.ncell <= 0) return 0;
  int dev = 0, nsm = 0;
  PGB_CUDA(cudaGetDevice(&dev));
  PGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (mapping == 1)
    return fp64 ? launch_newton_matrix_jr<M, double>(p, s, nsm) : launch_newton_matrix_jr<M, float>(p, s, nsm);
  if constexpr (THREAD) {
    return fp64 ? launch_newton_matrix_thread_jr<M, double>(p, s, nsm)
                : launch_newton_matrix_thread_jr<M, float>(p, s, nsm);
  } else {
    return set_err("newton matrix: mechanism %s has no cell-per-thread kernels", M::NAME);
  }
}

template <class M>
int heat_release_entry(const pgb_box* b, const pgb_array4* T, const pgb_array4* rhoYdot, const pgb_array4* hr,
                       cudaStream_t s) {
  if (check_arr(*T, *b, 1, "T", 0) || check_arr(*rhoYdot, *b, M::NS, "rhoYdot", 0) ||
      check_arr(*hr, *b, 1, "hr", 0))
    return -1;
  pgb::PointParams p;
  std::memset(&p, 0, sizeof(p));
  p.lo0 = b->lo[0]; p.lo1 = b->lo[1]; p.lo2 = b->lo[2];
  p.len0 = b->hi[0] - b->lo[0] + 1; p.len1 = b->hi[1] - b->lo[1] + 1; p.len2 = b->hi[2] - b->lo[2] + 1;
  p.T = arr_dev(*T); p.rY = arr_dev(*rhoYdot); p.out = arr_dev(*hr);
  const long long n = (long long)p.len0 * p.len1 * p.len2;
  if (n <= 0) return 0;
  pgb::heat_release_kernel<M><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(p);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

template <class M>
int h2t_entry(const pgb_box_view* v, double tmin, double tmax, cudaStream_t s) {
  const pgb_box& b = v->box;
  if (check_arr(v->rY, b, M::NS, "rY", 0) || check_arr(v->T, b, 1, "T", 0) ||
      check_arr(v->rEner, b, 1, "rEner", 0))
    return -1;
  pgb::PointParams p;
  p.lo0 = b.lo[0]; p.lo1 = b.lo[1]; p.lo2 = b.lo[2];
  p.len0 = b.hi[0] - b.lo[0] + 1; p.len1 = b.hi[1] - b.lo[1] + 1; p.len2 = b.hi[2] - b.lo[2] + 1;
  p.rY = arr_dev(v->rY); p.rE = arr_dev(v->rEner); p.T = arr_dev(v->T);
  p.tmin = tmin; p.tmax = tmax;
  const long long n = (long long)p.len0 * p.len1 * p.len2;
  if (n == 0) return 0;
  pgb::h2t_kernel<M><<<(unsigned)((n + 127) / 128), 128, 0, s>>>(p);
  PGB_CUDA(cudaGetLastError());
  return 0;
}

#define PGB_MECH_ENTRY(M)                                                                    \
  ::pgb_host::MechEntry {                                                                    \
    M::NAME, M::NS, M::NR, ::pgb_host::launch_bdf<M, float>, ::pgb_host::launch_bdf<M, double>, \
        ::pgb_host::launch_null<M>, pgb::bdf_smem_per_thread<M, float>(),                    \
        pgb::bdf_smem_per_thread<M, double>(),                                               \
        pgb::bdf_smem_per_thread<M, float, pgb::LAYOUT_Z_GLOBAL>(),                          \
        pgb::bdf_smem_per_thread<M, double, pgb::LAYOUT_Z_GLOBAL>(),                         \
        pgb::bdf_smem_per_thread<M, float, 3>(), pgb::bdf_smem_per_thread<M, double, 3>(),   \
        ::pgb_host::rates_entry<M>,                                                          \
        ::pgb_host::h2t_entry<M>, ::pgb_host::launch_surrogate<M>,                           \
        ::pgb_host::launch_surrogate_audit<M>, ::pgb_host::launch_bdf_warp<M, float>,        \
        ::pgb_host::launch_bdf_warp<M, double>, pgb::bdf_warp_smem_per_warp<M, float>(),     \
        pgb::bdf_warp_smem_per_warp<M, double>(), ::pgb_host::launch_surrogate_features<M>,  \
    {                                                                                        \
      ::pgb_host::warp_wpb_choice<M>(0), ::pgb_host::warp_wpb_choice<M>(1),                  \
          ::pgb_host::warp_wpb_choice<M>(2), ::pgb_host::warp_wpb_choice<M>(3)               \
    }                                                                                        \
    , ::pgb_host::heat_release_entry<M>, nullptr, nullptr, nullptr, nullptr,                \
        ::pgb_host::newton_matrix_entry<M, true>                                             \
  }

// Mechanisms whose cells also run group-per-cell (the 21-species size): all of the above plus
// the group kernel in both precisions.
#define PGB_MECH_ENTRY_GROUP(M)                                                              \
  ::pgb_host::MechEntry {                                                                    \
    M::NAME, M::NS, M::NR, ::pgb_host::launch_bdf<M, float>, ::pgb_host::launch_bdf<M, double>, \
        ::pgb_host::launch_null<M>, pgb::bdf_smem_per_thread<M, float>(),                    \
        pgb::bdf_smem_per_thread<M, double>(),                                               \
        pgb::bdf_smem_per_thread<M, float, pgb::LAYOUT_Z_GLOBAL>(),                          \
        pgb::bdf_smem_per_thread<M, double, pgb::LAYOUT_Z_GLOBAL>(),                         \
        pgb::bdf_smem_per_thread<M, float, 3>(), pgb::bdf_smem_per_thread<M, double, 3>(),   \
        ::pgb_host::rates_entry<M>,                                                          \
        ::pgb_host::h2t_entry<M>, ::pgb_host::launch_surrogate<M>,                           \
        ::pgb_host::launch_surrogate_audit<M>, ::pgb_host::launch_bdf_warp<M, float>,        \
        ::pgb_host::launch_bdf_warp<M, double>, pgb::bdf_warp_smem_per_warp<M, float>(),     \
        pgb::bdf_warp_smem_per_warp<M, double>(), ::pgb_host::launch_surrogate_features<M>,  \
    {                                                                                        \
      ::pgb_host::warp_wpb_choice<M>(0), ::pgb_host::warp_wpb_choice<M>(1),                  \
          ::pgb_host::warp_wpb_choice<M>(2), ::pgb_host::warp_wpb_choice<M>(3)               \
    }                                                                                        \
    , ::pgb_host::heat_release_entry<M>, ::pgb_host::launch_bdf_group<M, float>,             \
        ::pgb_host::launch_bdf_group<M, double>, ::pgb_host::group_cells_per_block<M, float>, \
        ::pgb_host::group_cells_per_block<M, double>,                                        \
        ::pgb_host::newton_matrix_entry<M, true>                                             \
  }

// Mechanisms too large for one cell per thread: warp-per-cell BDF, ReactorNull and T(h, Y) only.
#define PGB_MECH_ENTRY_WARP(M)                                                               \
  ::pgb_host::MechEntry {                                                                    \
    M::NAME, M::NS, M::NR, nullptr, nullptr, ::pgb_host::launch_null<M>, 0, 0, 0, 0, 0, 0,    \
        nullptr, ::pgb_host::h2t_entry<M>, nullptr, nullptr,                                 \
        ::pgb_host::launch_bdf_warp<M, float>, ::pgb_host::launch_bdf_warp<M, double>,       \
        pgb::bdf_warp_smem_per_warp<M, float>(), pgb::bdf_warp_smem_per_warp<M, double>(),   \
        nullptr,                                                                             \
    {                                                                                        \
      ::pgb_host::warp_wpb_choice<M>(0), ::pgb_host::warp_wpb_choice<M>(1),                  \
          ::pgb_host::warp_wpb_choice<M>(2), ::pgb_host::warp_wpb_choice<M>(3)               \
    }                                                                                        \
    , ::pgb_host::heat_release_entry<M>, nullptr, nullptr, nullptr, nullptr,                \
        ::pgb_host::newton_matrix_entry<M, false>                                            \
  }

// Converts and validates one box view into its device descriptor; cell numbering of the box
// starts at cell_offset.
inline int fill_box_dev(const pgb_box_view& v, int ns, long long cell_offset, int ibox,
                        pgb::BoxDev& d) {
  const pgb_box& bx = v.box;
  for (int k = 0; k < 3; ++k)
    if (bx.hi[k] < bx.lo[k]) return set_err("box %d is empty in dim %d", ibox, k);
  if (check_arr(v.rY, bx, ns, "rY", ibox) || check_arr(v.rY_src, bx, ns, "rY_src", ibox) ||
      check_arr(v.T, bx, 1, "T", ibox) || check_arr(v.rEner, bx, 1, "rEner", ibox) ||
      check_arr(v.rEner_src, bx, 1, "rEner_src", ibox) || check_arr(v.FC, bx, 1, "FC", ibox))
    return -1;
  if (v.mask.p && check_arr(v.mask, bx, 1, "mask", ibox)) return -1;
  std::memset(&d, 0, sizeof(d));
  d.sY_in = d.sE_in = d.sY_out = d.sE_out = 1.0;
  d.lo0 = bx.lo[0]; d.lo1 = bx.lo[1]; d.lo2 = bx.lo[2];
  d.len0 = bx.hi[0] - bx.lo[0] + 1;
  d.len1 = bx.hi[1] - bx.lo[1] + 1;
  d.len2 = bx.hi[2] - bx.lo[2] + 1;
  d.cell_offset = cell_offset;
  d.rY = arr_dev(v.rY);
  d.rYsrc = arr_dev(v.rY_src);
  d.T = arr_dev(v.T);
  d.rE = arr_dev(v.rEner);
  d.rEsrc = arr_dev(v.rEner_src);
  d.FC = arr_dev(v.FC);
  d.mask.p = static_cast<const int*>(v.mask.p);
  d.mask.jstride = v.mask.jstride;
  d.mask.kstride = v.mask.kstride;
  d.mask.begin0 = v.mask.begin[0];
  d.mask.begin1 = v.mask.begin[1];
  d.mask.begin2 = v.mask.begin[2];
  return 0;
}

// Registry lookup by mechanism name (nullptr when the mechanism is not compiled in).
const MechEntry* find_mech_entry(const char* name);

}  // namespace pgb_host

#endif  // PGB_REACTOR_REGISTRY_CUH
