// Allocation-free multi-box advance (pgb_react_boxes_noalloc).
//
// Some callers cannot allocate device memory when they call the reactor: PeleLM runs on an AMReX
// arena that reserves most of the GPU at start-up, so a library cudaMalloc at react() time can
// fail or fragment what the arena left, and cudaMalloc / cudaFree may synchronize the device in
// the middle of a time step. This entry point therefore takes every buffer from the caller
// (inputs and outputs, through the box views) and keeps its own scratch — the box table, the
// work-queue head and the counters — in one fixed file-scope device array below. It calls no
// cudaMalloc, cudaFree or other allocating routine; it launches the same persistent
// work-stealing kernels as pgb_reactor_react_boxes (cell per thread for small mechanisms, cell
// per warp for the larger ones), with their working state in shared memory only.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cstring>

#include "reactor_registry.cuh"

namespace {

using namespace pgb_host;

struct NoAllocScratch {
  pgb::BoxDev boxes[PGB_NOALLOC_MAX_BOXES];
  unsigned long long next_cell;
  pgb::ReactStats stats;
};

// The scratch of every call on a device (about 370 KB for 1024 boxes). Every GPU that loads
// the library holds one copy until the process exits. Host code must never use this name as
// a device address: it only names the symbol for cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[sizeof(NoAllocScratch)];

constexpr int kMaxDevices = 64;
// Device address of g_noalloc_scratch per device, resolved on that device's first call.
std::atomic<NoAllocScratch*> g_scratch_addr[kMaxDevices];

int scratch_of_current_device(NoAllocScratch** out) {
  int dev = 0;
  PGB_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= kMaxDevices) return set_err("device ordinal %d out of range", dev);
  NoAllocScratch* p = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!p) {
    void* addr = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&addr, g_noalloc_scratch);
    if (e != cudaSuccess || !addr)
      return set_err("cudaGetSymbolAddress(noalloc scratch) failed on device %d: %s", dev,
                     cudaGetErrorString(e));
    p = static_cast<NoAllocScratch*>(addr);
    g_scratch_addr[dev].store(p, std::memory_order_release);
  }
  *out = p;
  return 0;
}

// Box descriptors travel to the scratch array as kernel parameters, kBoxesPerCopy at a time
// (3.5 KB, under the classic 4 KB parameter limit): the launch copies them, so no host buffer
// has to outlive the call and nothing pageable is referenced by the stream.
constexpr int kBoxesPerCopy = 8;
struct BoxChunk {
  pgb::BoxDev b[kBoxesPerCopy];
};
static_assert(sizeof(BoxChunk) <= 4000, "box chunk exceeds the kernel parameter space");

__global__ void store_boxes_kernel(const BoxChunk chunk, int n, pgb::BoxDev* dst) {
  constexpr int kWords = (int)(sizeof(pgb::BoxDev) / sizeof(unsigned long long));
  static_assert(sizeof(pgb::BoxDev) % sizeof(unsigned long long) == 0, "BoxDev is not 8-byte sized");
  const unsigned long long* src = reinterpret_cast<const unsigned long long*>(chunk.b);
  unsigned long long* out = reinterpret_cast<unsigned long long*>(dst);
  for (int i = threadIdx.x; i < n * kWords; i += blockDim.x) out[i] = src[i];
}

}  // namespace

extern "C" int pgb_react_boxes_noalloc(const char* mechanism, const pgb_box_view* views, int nbox,
                                       double dt_react, double rtol, double atol, int max_order,
                                       int max_steps, int fp64, void* stream, pgb_stats* stats) {
  const MechEntry* m = find_mech_entry(mechanism);
  if (!m) return set_err("unknown mechanism '%s'", mechanism ? mechanism : "(null)");
  if (nbox < 1 || !views) return set_err("noalloc: need at least one box view");
  if (nbox > PGB_NOALLOC_MAX_BOXES)
    return set_err("noalloc: %d boxes exceed the fixed scratch capacity of %d boxes; split the "
                   "call or use pgb_reactor_react_boxes", nbox, PGB_NOALLOC_MAX_BOXES);
  if (!(dt_react > 0.0) || !(rtol > 0.0) || !(atol > 0.0))
    return set_err("noalloc: dt_react, rtol and atol must be > 0");
  if (max_order < 1 || max_order > pgb::QMAX) return set_err("noalloc: max_order must be in [1, %d]", pgb::QMAX);
  if (max_steps < 1) return set_err("noalloc: max_steps must be >= 1");
  // Kernel choice, all state in shared memory: cell per thread where 64 threads' state fits a
  // block (the LiDryer-sized mechanisms), else cell per warp with the most preferred compiled
  // warps-per-block size that fits (drm19- and GRI-sized).
  const int per_thread = fp64 ? m->smem_fp64 : m->smem_mixed;
  const bool thread_ok = m->bdf_mixed && m->ns <= 12 && per_thread * 64 <= kMaxSmemPerBlock;
  int wpb = 0;
  if (!thread_ok) {
    const int per_warp = fp64 ? m->wsmem_fp64 : m->wsmem_mixed;
    for (int i = 0; i < 4 && m->wpb_choice[i] > 0 && !wpb; ++i)
      if (m->wpb_choice[i] * per_warp <= kMaxSmemPerBlock) wpb = m->wpb_choice[i];
    if (!wpb || !m->warp_mixed)
      return set_err("noalloc: no compiled kernel of mechanism '%s' keeps its state in shared memory", m->name);
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  // Under stream capture the call records only stream work (box-table kernels, memsets, the
  // advance); stats need a wait for the advance, which a capture cannot contain.
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  PGB_CUDA(cudaStreamIsCapturing(st, &cap));
  if (cap != cudaStreamCaptureStatusNone && stats)
    return set_err("noalloc: stats wait for the advance, which a stream capture cannot contain; "
                   "pass stats = NULL while capturing");
  NoAllocScratch* S = nullptr;
  if (scratch_of_current_device(&S)) return -1;

  // Box table: validated and converted here, copied into the scratch array through kernel
  // parameters.
  BoxChunk chunk;
  long long ncell = 0;
  for (int b0 = 0; b0 < nbox; b0 += kBoxesPerCopy) {
    const int n = (nbox - b0 < kBoxesPerCopy) ? nbox - b0 : kBoxesPerCopy;
    for (int i = 0; i < n; ++i) {
      const pgb_box_view& v = views[b0 + i];
      if (fill_box_dev(v, m->ns, ncell, b0 + i, chunk.b[i])) return -1;
      ncell += (long long)chunk.b[i].len0 * chunk.b[i].len1 * chunk.b[i].len2;
    }
    store_boxes_kernel<<<1, 128, 0, st>>>(chunk, n, &S->boxes[b0]);
    PGB_CUDA(cudaGetLastError());
  }
  // The scratch keeps the previous call's contents: the queue head and counters restart at 0.
  PGB_CUDA(cudaMemsetAsync(&S->next_cell, 0, sizeof(S->next_cell), st));
  PGB_CUDA(cudaMemsetAsync(&S->stats, 0, sizeof(S->stats), st));

  pgb::ReactParams p;
  std::memset(&p, 0, sizeof(p));
  p.boxes = S->boxes;
  p.nbox = nbox;
  p.ncell = ncell;
  p.dt = dt_react;
  p.rtol = rtol;
  for (int i = 0; i < pgb::MAXN; ++i) p.atol[i] = atol;
  p.max_order = max_order;
  p.max_steps = max_steps;
  p.next_cell = &S->next_cell;
  p.stats = &S->stats;
  p.lu_scratch = nullptr;  // Jacobian/LU slices and Nordsieck histories stay in shared memory
  p.z_scratch = nullptr;
  p.cell_list = nullptr;
  p.ncell_dev = nullptr;
  p.retry_list = nullptr;  // a failed cell keeps its state at failure and FC = -status
  p.retry_count = nullptr;
  int dev = 0, nsm = 0;
  PGB_CUDA(cudaGetDevice(&dev));
  PGB_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  if (ncell > 0) {
    if (thread_ok) {
      const int tpb = (per_thread * 128 <= kMaxSmemPerBlock) ? 128 : 64;
      const long long nblocks = std::min<long long>((ncell + tpb - 1) / tpb, nsm);
      const LaunchFn fn = fp64 ? m->bdf_fp64 : m->bdf_mixed;
      if (fn(p, tpb, st, (int)nblocks)) return -1;
    } else {
      const long long nblocks = std::min<long long>((ncell + wpb - 1) / wpb, nsm);
      const LaunchFn fn = fp64 ? m->warp_fp64 : m->warp_mixed;
      if (fn(p, wpb, st, (int)nblocks)) return -1;
    }
  }
  if (stats) {
    pgb::ReactStats h;
    PGB_CUDA(cudaMemcpyAsync(&h, &S->stats, sizeof(h), cudaMemcpyDeviceToHost, st));
    PGB_CUDA(cudaStreamSynchronize(st));
    stats->ncell = (unsigned long long)ncell;
    stats->nst = h.nst; stats->nfe = h.nfe; stats->nje = h.nje; stats->netf = h.netf;
    stats->ncfn = h.ncfn; stats->nfail = h.nfail; stats->max_nst = h.max_nst;
    for (int i = 0; i < 16; ++i) stats->hist[i] = h.hist[i];
    stats->nretry = h.nretry;
  }
  return 0;
}
