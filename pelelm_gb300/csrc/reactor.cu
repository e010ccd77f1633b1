// Host driver and C ABI of the GB300 reactor (include/pelelm_gb300.h).
//
// Stands in for the PelePhysics ReactorBase implementations that PeleLM reaches through
// m_reactor (Source/PeleLM.H:673-674): create/init (Source/PeleLM.cpp:706-709),
// set_typ_vals_ode (:1513), react (:5752) and close (:930), plus a multi-box entry point that
// advances every box of every level in one persistent launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#include "reactor_registry.cuh"
#include "surrogate_host.h"

namespace pgb_host {

namespace {
thread_local std::string g_err;
}

int set_err(const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof(buf), fmt, ap);
  va_end(ap);
  g_err = buf;
  return -1;
}

}  // namespace pgb_host

#include "gen/mech_registry.inc"

using namespace pgb_host;

namespace {

// ------------------------------------------------------------------ options
struct Options {
  double rtol = 1e-6;
  double atol = 1e-10;
  int max_order = 5;
  int max_steps = 20000;
  bool use_typ_vals = false;
  bool mixed = true;       // gb.precision = mixed (FP32 J/LU) | fp64
  int tpb = 0;             // 0 = default per mechanism
  bool graph = false;
  int z_global = -1;       // gb.history = shared | global (L2-resident Nordsieck); -1 = auto
  int lu_global = -1;      // gb.lu = shared | global (L2-resident Jacobian/LU); -1 = auto
  int mapping = -1;        // gb.mapping = thread | warp | group (cell per thread / warp / lane group); -1 = auto
  int group = 8;           // gb.group: lanes per cell of the group mapping (4 or 8)
  int wpb = 0;             // gb.wpb: warps per block of the warp mapping (0 = most that fit)
  bool autotune = false;   // gb.autotune: time the compiled mappings on the first advance's cells
  bool retry = true;       // gb.retry: cells the mixed-precision pass fails are integrated again in FP64
  std::string solve_type = "denseAJ_direct";
  int analytical_jacobian = 1;
  std::string surrogate;   // gb.surrogate = trained surrogate file: surrogate + BDF fallback
  SgOverrides sg;          // gb.sg.* threshold overrides
  unsigned long long sg_seed = 1;
};

int parse_options(const char* s, Options& o) {
  if (!s) return 0;
  std::string str(s);
  for (char& c : str)
    if (c == ';' || c == ',' || c == '\n' || c == '\t') c = ' ';
  std::istringstream is(str);
  std::string tok;
  while (is >> tok) {
    const size_t eq = tok.find('=');
    if (eq == std::string::npos) return set_err("option '%s' is not key=value", tok.c_str());
    const std::string k = tok.substr(0, eq), v = tok.substr(eq + 1);
    try {
      if (k == "ode.rtol") o.rtol = std::stod(v);
      else if (k == "ode.atol") o.atol = std::stod(v);
      else if (k == "cvode.max_order") o.max_order = std::stoi(v);
      else if (k == "ode.max_steps") o.max_steps = std::stoi(v);
      else if (k == "peleLM.use_typ_vals_chem") o.use_typ_vals = std::stoi(v) != 0;
      else if (k == "cvode.solve_type") o.solve_type = v;
      else if (k == "ode.analytical_jacobian") o.analytical_jacobian = std::stoi(v);
      else if (k == "gb.precision") {
        if (v == "mixed") o.mixed = true;
        else if (v == "fp64") o.mixed = false;
        else return set_err("gb.precision must be mixed or fp64, got '%s'", v.c_str());
      } else if (k == "gb.tpb") o.tpb = std::stoi(v);
      else if (k == "gb.graph") o.graph = std::stoi(v) != 0;
      else if (k == "gb.mapping") {
        if (v == "thread") o.mapping = 0;
        else if (v == "warp") o.mapping = 1;
        else if (v == "group") o.mapping = 2;
        else return set_err("gb.mapping must be thread, warp or group, got '%s'", v.c_str());
      } else if (k == "gb.group") {
        o.group = std::stoi(v);
        if (o.group != 4 && o.group != 8) return set_err("gb.group must be 4 or 8, got '%s'", v.c_str());
      } else if (k == "gb.wpb") o.wpb = std::stoi(v);
      else if (k == "gb.autotune") o.autotune = std::stoi(v) != 0;
      else if (k == "gb.retry") o.retry = std::stoi(v) != 0;
      else if (k == "gb.surrogate") o.surrogate = v;
      else if (k == "gb.sg.audit") o.sg.audit_frac = std::stod(v);
      else if (k == "gb.sg.mis") o.sg.mis = std::stod(v);
      else if (k == "gb.sg.cons") o.sg.cons = std::stod(v);
      else if (k == "gb.sg.disT") o.sg.disT = std::stod(v);
      else if (k == "gb.sg.disY") o.sg.disY = std::stod(v);
      else if (k == "gb.sg.neg") o.sg.neg = std::stod(v);
      else if (k == "gb.sg.ood_margin") o.sg.ood_margin = std::stod(v);
      else if (k == "gb.sg.tol_T") o.sg.tol_T = std::stod(v);
      else if (k == "gb.sg.tol_Y") o.sg.tol_Y = std::stod(v);
      else if (k == "gb.sg.models") o.sg.models = std::stoi(v);
      else if (k == "gb.sg.seed") o.sg_seed = std::stoull(v);
      else if (k == "gb.history" || k == "gb.lu") {
        int& f = (k == "gb.history") ? o.z_global : o.lu_global;
        if (v == "global") f = 1;
        else if (v == "shared") f = 0;
        else return set_err("%s must be global or shared, got '%s'", k.c_str(), v.c_str());
      }
      else return set_err("unknown option '%s'", k.c_str());
    } catch (...) {
      return set_err("bad value for option '%s': '%s'", k.c_str(), v.c_str());
    }
  }
  if (!(o.rtol > 0.0) || !(o.atol > 0.0)) return set_err("ode.rtol and ode.atol must be > 0");
  if (o.max_order < 1 || o.max_order > pgb::QMAX)
    return set_err("cvode.max_order must be in [1, %d]", pgb::QMAX);
  if (o.max_steps < 1) return set_err("ode.max_steps must be >= 1");
  // Every accepted linear-solver key runs the dense direct Newton solve with the analytic
  // Jacobian. The matrix-free Krylov keys of the reference's GPU decks (cvode.solve_type = GMRES,
  // Exec/RegTests/FlameSheet/inputs.3d-regt_GPU:88) map to it too: GMRES solves the same Newton
  // system (I - gamma J) x = r only to a fraction of the Newton tolerance, the direct solve
  // exactly, and the nonlinear iteration's convergence test (and with it rtol/atol) is unchanged.
  static const char* const kDense[] = {"denseAJ_direct", "dense_direct", "dense", "denseFDJ_direct"};
  static const char* const kKrylov[] = {"GMRES", "precGMRES"};
  bool known = false;
  for (const char* k : kDense) known = known || o.solve_type == k;
  for (const char* k : kKrylov) known = known || o.solve_type == k;
  if (!known)
    return set_err("cvode.solve_type '%s' is not provided (dense direct: denseAJ_direct, "
                   "dense_direct, dense, denseFDJ_direct; GMRES and precGMRES run the dense direct "
                   "solve)", o.solve_type.c_str());
  return 0;
}

const MechEntry* find_mech(const char* name);

int build_boxes(const pgb_box_view* v, int nbox, int ns, std::vector<pgb::BoxDev>& out,
                long long& ncell) {
  out.resize(nbox);
  ncell = 0;
  for (int b = 0; b < nbox; ++b) {
    const pgb_box& bx = v[b].box;
    for (int d = 0; d < 3; ++d)
      if (bx.hi[d] < bx.lo[d]) return set_err("box %d is empty in dim %d", b, d);
    if (check_arr(v[b].rY, bx, ns, "rY", b) || check_arr(v[b].rY_src, bx, ns, "rY_src", b) ||
        check_arr(v[b].T, bx, 1, "T", b) || check_arr(v[b].rEner, bx, 1, "rEner", b) ||
        check_arr(v[b].rEner_src, bx, 1, "rEner_src", b) || check_arr(v[b].FC, bx, 1, "FC", b))
      return -1;
    if (v[b].mask.p && check_arr(v[b].mask, bx, 1, "mask", b)) return -1;
    pgb::BoxDev& d = out[b];
    std::memset(&d, 0, sizeof(d));  // also the padding: the graph cache compares box tables bytewise
    d.sY_in = d.sE_in = d.sY_out = d.sE_out = 1.0;
    d.lo0 = bx.lo[0]; d.lo1 = bx.lo[1]; d.lo2 = bx.lo[2];
    d.len0 = bx.hi[0] - bx.lo[0] + 1;
    d.len1 = bx.hi[1] - bx.lo[1] + 1;
    d.len2 = bx.hi[2] - bx.lo[2] + 1;
    d.cell_offset = ncell;
    ncell += (long long)d.len0 * d.len1 * d.len2;
    d.rY = arr_dev(v[b].rY);
    d.rYsrc = arr_dev(v[b].rY_src);
    d.T = arr_dev(v[b].T);
    d.rE = arr_dev(v[b].rEner);
    d.rEsrc = arr_dev(v[b].rEner_src);
    d.FC = arr_dev(v[b].FC);
    d.mask.p = static_cast<const int*>(v[b].mask.p);
    d.mask.jstride = v[b].mask.jstride;
    d.mask.kstride = v[b].mask.kstride;
    d.mask.begin0 = v[b].mask.begin[0];
    d.mask.begin1 = v[b].mask.begin[1];
    d.mask.begin2 = v[b].mask.begin[2];
  }
  return 0;
}

// ------------------------------------------------------------------ per-stream scratch
struct Scratch {
  pgb::BoxDev* d_boxes = nullptr;
  size_t box_cap = 0;
  pgb::BoxDev* h_boxes = nullptr;  // pinned staging
  unsigned long long* d_counter = nullptr;
  void* d_z = nullptr;             // Nordsieck histories of the resident threads
  size_t z_cap = 0;
  void* d_lu = nullptr;            // Jacobian/LU slices of the resident threads
  size_t lu_cap = 0;
  pgb::ReactStats* d_stats = nullptr;
  // surrogate: fallback cell list, audit records, counters
  void* d_fallback = nullptr;
  size_t fallback_cap = 0;
  void* d_audit = nullptr;
  size_t audit_cap = 0;
  unsigned long long* d_sg_counts = nullptr;  // fallback count, audit count, seed
  pgb::SurrogateStats* d_sg_stats = nullptr;
  // cells the mixed-precision pass failed, integrated again by the FP64 pass
  void* d_retry = nullptr;
  size_t retry_cap = 0;
  unsigned long long* d_retry_count = nullptr;
  cudaEvent_t done = nullptr;
  long long last_ncell = 0;
  // graph cache
  cudaGraphExec_t gexec = nullptr;
  std::vector<pgb::BoxDev> gkey;
  double gdt = -1.0;
};

}  // namespace

struct pgb_reactor {
  std::string name;
  const MechEntry* mech = nullptr;
  Options opt;
  bool null_reactor = false;
  std::vector<double> typ;
  std::mutex mu;
  std::map<cudaStream_t, Scratch> scratch;
  cudaStream_t last_stream = nullptr;
  int device = 0, nsm = 0;
  SgModel sg;  // loaded when options name a surrogate file
  bool tuned = false;
  std::string tuning;  // autotuner report
};

namespace {

void free_scratch(Scratch& s) {
  if (s.gexec) cudaGraphExecDestroy(s.gexec);
  if (s.d_boxes) cudaFree(s.d_boxes);
  if (s.h_boxes) cudaFreeHost(s.h_boxes);
  if (s.d_counter) cudaFree(s.d_counter);
  if (s.d_stats) cudaFree(s.d_stats);
  if (s.d_z) cudaFree(s.d_z);
  if (s.d_lu) cudaFree(s.d_lu);
  if (s.d_fallback) cudaFree(s.d_fallback);
  if (s.d_audit) cudaFree(s.d_audit);
  if (s.d_sg_counts) cudaFree(s.d_sg_counts);
  if (s.d_sg_stats) cudaFree(s.d_sg_stats);
  if (s.d_retry) cudaFree(s.d_retry);
  if (s.d_retry_count) cudaFree(s.d_retry_count);
  if (s.done) cudaEventDestroy(s.done);
  s = Scratch();
}

int ensure_scratch(pgb_reactor* r, cudaStream_t st, size_t nbox, Scratch** out) {
  Scratch& s = r->scratch[st];
  if (!s.d_counter) {
    PGB_CUDA(cudaMalloc(&s.d_counter, sizeof(unsigned long long)));
    PGB_CUDA(cudaMalloc(&s.d_stats, sizeof(pgb::ReactStats)));
    PGB_CUDA(cudaMalloc(&s.d_retry_count, sizeof(unsigned long long)));
    PGB_CUDA(cudaEventCreateWithFlags(&s.done, cudaEventDisableTiming));
    if (r->sg.d_net) {
      PGB_CUDA(cudaMalloc(&s.d_sg_counts, 3 * sizeof(unsigned long long)));
      PGB_CUDA(cudaMalloc(&s.d_sg_stats, sizeof(pgb::SurrogateStats)));
      const unsigned long long seed = r->opt.sg_seed;
      PGB_CUDA(cudaMemcpy(s.d_sg_counts + 2, &seed, sizeof(seed), cudaMemcpyHostToDevice));
    }
  }
  if (nbox > s.box_cap) {
    if (s.done) PGB_CUDA(cudaEventSynchronize(s.done));
    if (s.gexec) { cudaGraphExecDestroy(s.gexec); s.gexec = nullptr; s.gkey.clear(); }
    if (s.d_boxes) PGB_CUDA(cudaFree(s.d_boxes));
    if (s.h_boxes) PGB_CUDA(cudaFreeHost(s.h_boxes));
    size_t cap = std::max<size_t>(nbox, 64);
    PGB_CUDA(cudaMalloc(&s.d_boxes, cap * sizeof(pgb::BoxDev)));
    PGB_CUDA(cudaMallocHost(&s.h_boxes, cap * sizeof(pgb::BoxDev)));
    s.box_cap = cap;
  }
  *out = &s;
  return 0;
}

bool same_boxes(const std::vector<pgb::BoxDev>& a, const pgb::BoxDev* b, size_t n) {
  return a.size() == n && std::memcmp(a.data(), b, n * sizeof(pgb::BoxDev)) == 0;
}

// Threads per block and grid of the persistent launch, and the global Nordsieck scratch it
// needs (0 when the histories live in shared memory).
struct LaunchPlan {
  int tpb = 128, nblocks = 1;
  bool z_global = false, lu_global = false;
  size_t z_bytes = 0, lu_bytes = 0;
  bool warp = false;   // warp-per-cell kernel; tpb then holds warps per block
  bool group = false;  // group-per-cell kernel; tpb then holds lanes per cell
};

int mapping_of(const pgb_reactor* r);

// First layout (all shared; global Nordsieck history; global history and LU) whose shared
// footprint fits 128 threads per block (the occupancy that measures best), unless options
// force the layout or the block size. `mixed` selects the precision planned for (the FP64
// retry pass plans FP64 whatever gb.precision says, and then ignores a gb.wpb that does not
// fit FP64's shared memory).
LaunchPlan plan_launch(const pgb_reactor* r, long long ncell, bool mixed) {
  LaunchPlan pl;
  const MechEntry& m = *r->mech;
  if (mapping_of(r) == 2) {
    // lane groups per cell: as many warps per block as fit shared memory, one block per SM
    const int G = r->opt.group;
    const int per_block = (mixed ? m.group_cells_mixed : m.group_cells_fp64)(G);
    pl.group = true;
    pl.tpb = G;
    pl.nblocks = (int)std::min<long long>(r->nsm, std::max<long long>(1, (ncell + per_block - 1) / std::max(per_block, 1)));
    return pl;
  }
  if (mapping_of(r) == 1) {
    // warp per cell: as many warps per block as fit shared memory (or gb.wpb), one block per SM
    const int per = mixed ? m.wsmem_mixed : m.wsmem_fp64;
    int wpb = r->opt.wpb;
    if (wpb > 0 && mixed != r->opt.mixed && wpb * per > kMaxSmemPerBlock) wpb = 0;
    if (wpb <= 0) {  // most preferred compiled size whose shared memory fits
      for (int i = 0; i < 4 && m.wpb_choice[i] > 0; ++i) {
        wpb = m.wpb_choice[i];
        if (m.wpb_choice[i] * per <= kMaxSmemPerBlock) break;
      }
    }
    pl.warp = true;
    pl.tpb = wpb;
    pl.nblocks = (int)std::min<long long>(r->nsm, std::max<long long>(1, (ncell + wpb - 1) / wpb));
    return pl;
  }
  const int per[3] = {mixed ? m.smem_mixed : m.smem_fp64, mixed ? m.smem_mixed_g : m.smem_fp64_g,
                      mixed ? m.smem_mixed_gl : m.smem_fp64_gl};
  const int tpb = r->opt.tpb > 0 ? r->opt.tpb : 128;
  int choice = -1;
  for (int c = 0; c < 3 && choice < 0; ++c) {
    const bool zg = c >= 1, lg = c >= 2;
    if (r->opt.z_global >= 0 && (r->opt.z_global == 1) != zg) continue;
    if (r->opt.lu_global >= 0 && (r->opt.lu_global == 1) != lg) continue;
    if (per[c] * tpb <= kMaxSmemPerBlock) choice = c;
  }
  if (choice < 0) choice = 2;  // the launch reports the shared-memory shortfall
  pl.tpb = tpb;
  pl.z_global = choice >= 1;
  pl.lu_global = choice >= 2;
  // persistent grid: one CTA per SM, never more CTAs than there are blocks' worth of cells
  const long long max_blocks = std::max<long long>(1, (ncell + pl.tpb - 1) / pl.tpb);
  pl.nblocks = (int)std::min<long long>(r->nsm, max_blocks);
  const int N = m.ns + 1;
  const size_t slots = (size_t)pl.nblocks * pl.tpb;
  if (pl.z_global) pl.z_bytes = slots * (pgb::QMAX + 2) * N * sizeof(double);
  if (pl.lu_global) pl.lu_bytes = slots * N * N * (mixed ? sizeof(float) : sizeof(double));
  return pl;
}

// Grows one global scratch buffer (outside any stream capture; captured graphs that point at
// the old buffer are dropped).
int ensure_buf(Scratch& s, void*& buf, size_t& cap, size_t bytes) {
  if (bytes <= cap) return 0;
  if (s.done) PGB_CUDA(cudaEventSynchronize(s.done));
  if (s.gexec) { cudaGraphExecDestroy(s.gexec); s.gexec = nullptr; s.gkey.clear(); }
  if (buf) PGB_CUDA(cudaFree(buf));
  buf = nullptr;
  cap = 0;
  PGB_CUDA(cudaMalloc(&buf, bytes));
  cap = bytes;
  return 0;
}

// Kernel mapping: 0 cell per thread, 1 cell per warp, 2 cell per lane group. Cell-per-thread
// kernels exist for mechanisms whose per-cell state fits a thread, group kernels for the
// 21-species size; gb.mapping overrides the default below.
int mapping_of(const pgb_reactor* r) {
  if (r->opt.mapping >= 0) return r->opt.mapping;
  if (!r->mech->bdf_mixed) return 1;
  // measured: cell per thread for the 9-species mechanism (4x faster than per warp); from the
  // 21-species one on the per-thread state no longer fits registers: lane groups where compiled,
  // else one warp per cell
  if (r->mech->ns <= 12) return 0;
  return r->mech->group_mixed ? 2 : 1;
}

// Audit records kept per call: twice the expected sample plus slack (cells past the capacity
// are simply not audited).
long long audit_capacity(const pgb_reactor* r, long long ncell) {
  if (!(r->sg.audit_frac > 0.0)) return 0;
  return std::min<long long>(ncell, (long long)(2.0 * r->sg.audit_frac * (double)ncell) + 1024);
}

int enqueue_advance(pgb_reactor* r, Scratch& s, int nbox, long long ncell, double dt,
                    cudaStream_t st) {
  pgb::ReactParams p;
  std::memset(&p, 0, sizeof(p));
  p.boxes = s.d_boxes;
  p.nbox = nbox;
  p.ncell = ncell;
  p.dt = dt;
  p.rtol = r->opt.rtol;
  const int N = r->mech->ns + 1;
  for (int i = 0; i < N; ++i)
    p.atol[i] = (r->opt.use_typ_vals && (int)r->typ.size() == N) ? r->opt.atol * r->typ[i] : r->opt.atol;
  p.max_order = r->opt.max_order;
  p.max_steps = r->opt.max_steps;
  p.next_cell = s.d_counter;
  p.stats = s.d_stats;
  PGB_CUDA(cudaMemcpyAsync(s.d_boxes, s.h_boxes, nbox * sizeof(pgb::BoxDev), cudaMemcpyHostToDevice, st));
  PGB_CUDA(cudaMemsetAsync(s.d_counter, 0, sizeof(unsigned long long), st));
  PGB_CUDA(cudaMemsetAsync(s.d_stats, 0, sizeof(pgb::ReactStats), st));
  if (ncell == 0) return 0;
  if (r->null_reactor) {
    const long long nb = std::min<long long>((ncell + 255) / 256, (long long)r->nsm * 8);
    return r->mech->null_fn(p, st, (int)nb);
  }
  const LaunchPlan pl = plan_launch(r, ncell, r->opt.mixed);
  p.lu_scratch = pl.lu_bytes ? s.d_lu : nullptr;
  p.z_scratch = pl.z_bytes ? s.d_z : nullptr;
  LaunchFn fn = pl.group ? (r->opt.mixed ? r->mech->group_mixed : r->mech->group_fp64)
               : pl.warp ? (r->opt.mixed ? r->mech->warp_mixed : r->mech->warp_fp64)
                         : (r->opt.mixed ? r->mech->bdf_mixed : r->mech->bdf_fp64);
  // mixed precision with retry: the cells its pass fails (FP32 Newton matrices can stall where
  // FP64 ones converge) are listed on the device and integrated again from their untouched
  // inputs by the FP64 kernel, on the same stream (and in the same graph)
  const bool retry = r->opt.mixed && r->opt.retry && s.d_retry && s.d_retry_count &&
                     (long long)(s.retry_cap / sizeof(long long)) >= ncell;
  if (retry) {
    p.retry_list = static_cast<long long*>(s.d_retry);
    p.retry_count = s.d_retry_count;
    PGB_CUDA(cudaMemsetAsync(s.d_retry_count, 0, sizeof(unsigned long long), st));
  }
  auto run_bdf = [&]() -> int {
    if (fn(p, pl.tpb, st, pl.nblocks)) return -1;
    if (!retry) return 0;
    const LaunchPlan p64 = plan_launch(r, ncell, false);
    pgb::ReactParams q = p;
    q.cell_list = p.retry_list;
    q.ncell_dev = p.retry_count;
    q.retry_list = nullptr;
    q.retry_count = nullptr;
    q.lu_scratch = p64.lu_bytes ? s.d_lu : nullptr;
    q.z_scratch = p64.z_bytes ? s.d_z : nullptr;
    PGB_CUDA(cudaMemsetAsync(s.d_counter, 0, sizeof(unsigned long long), st));
    const LaunchFn f64 = p64.group ? r->mech->group_fp64 : p64.warp ? r->mech->warp_fp64 : r->mech->bdf_fp64;
    return f64(q, p64.tpb, st, p64.nblocks);
  };
  if (!r->sg.d_net) return run_bdf();

  // surrogate for every cell; the cells it does not accept (and the audit sample) go to the
  // BDF through the device list, then the audit compares
  pgb::SurrogateParams sp;
  sp.boxes = s.d_boxes;
  sp.nbox = nbox;
  sp.ncell = ncell;
  sp.dt = dt;
  sp.net = r->sg.d_net;
  sp.fallback_list = static_cast<long long*>(s.d_fallback);
  sp.fallback_count = s.d_sg_counts;
  sp.audit_count = s.d_sg_counts + 1;
  sp.seed_dev = s.d_sg_counts + 2;
  sp.audit_cap = audit_capacity(r, ncell);
  sp.audit_cell = static_cast<long long*>(s.d_audit);
  sp.audit_pred = reinterpret_cast<double*>(static_cast<long long*>(s.d_audit) + sp.audit_cap);
  sp.stats = s.d_sg_stats;
  sp.raw_out = nullptr;
  sp.raw_in = nullptr;
  PGB_CUDA(cudaMemsetAsync(s.d_sg_counts, 0, 2 * sizeof(unsigned long long), st));
  PGB_CUDA(cudaMemsetAsync(s.d_sg_stats, 0, sizeof(pgb::SurrogateStats), st));
  const long long ntiles = (ncell + pgb::SG_TILE - 1) / pgb::SG_TILE;
  if (r->mech->sg_fn(sp, st, (int)std::min<long long>(ntiles, r->nsm))) return -1;
  p.cell_list = sp.fallback_list;
  p.ncell_dev = sp.fallback_count;
  if (run_bdf()) return -1;
  return r->mech->sg_audit_fn(sp, st, r->nsm);
}

}  // namespace

// ================================================================== C ABI
extern "C" {

int pgb_version(void) { return PGB_ABI_VERSION; }

int pgb_last_error(char* buf, size_t n) {
  if (buf && n) {
    std::strncpy(buf, g_err.c_str(), n - 1);
    buf[n - 1] = 0;
  }
  return (int)g_err.size();
}

int pgb_mechanism_info(const char* mechanism, int* ns, int* nr) {
  const MechEntry* m = find_mech(mechanism);
  if (!m) return set_err("unknown mechanism '%s'", mechanism ? mechanism : "(null)");
  if (ns) *ns = m->ns;
  if (nr) *nr = m->nr;
  return 0;
}

pgb_reactor* pgb_reactor_create(const char* name, const char* mechanism, int reactor_type,
                                const char* options) {
  std::string n = name ? name : "";
  if (n == "ReactorRK64" || n == "ReactorArkode") {
    set_err("reactor '%s' is not provided by this library (ReactorCvode, ReactorNull)", n.c_str());
    return nullptr;
  }
  if (n != "ReactorCvode" && n != "ReactorNull") {
    set_err("unknown reactor '%s'", n.c_str());
    return nullptr;
  }
  if (reactor_type != 2) {
    set_err("reactor_type %d not supported: only 2 (rho h, constant pressure) as PeleLM uses",
            reactor_type);
    return nullptr;
  }
  const MechEntry* m = find_mech(mechanism);
  if (!m) {
    set_err("unknown mechanism '%s'", mechanism ? mechanism : "(null)");
    return nullptr;
  }
  Options o;
  if (parse_options(options, o)) return nullptr;
  if (o.mapping == 0 && !m->bdf_mixed) {
    set_err("mechanism '%s' has no cell-per-thread kernel (gb.mapping=warp)", m->name);
    return nullptr;
  }
  if (o.mapping == 2 && !m->group_mixed) {
    set_err("mechanism '%s' has no group-per-cell kernel (gb.mapping=warp)", m->name);
    return nullptr;
  }
  if (!o.surrogate.empty() && !m->sg_fn) {
    set_err("no surrogate kernel is compiled for mechanism '%s'", m->name);
    return nullptr;
  }
  int dev = 0, nsm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) {
    set_err("no CUDA device available");
    return nullptr;
  }
  auto* r = new pgb_reactor();
  r->name = n;
  r->mech = m;
  r->opt = o;
  r->null_reactor = (n == "ReactorNull");
  r->device = dev;
  r->nsm = nsm;
  if (!o.surrogate.empty()) {
    if (r->null_reactor || sg_load(o.surrogate.c_str(), m->name, m->ns, o.sg, r->sg)) {
      if (r->null_reactor) set_err("gb.surrogate needs ReactorCvode (its fallback integrator)");
      delete r;
      return nullptr;
    }
  }
  return r;
}

int pgb_reactor_set_typ_vals_ode(pgb_reactor* r, const double* typ, int n) {
  if (!r) return set_err("null reactor");
  if (n != r->mech->ns + 1) return set_err("set_typ_vals_ode: expected %d values, got %d", r->mech->ns + 1, n);
  std::lock_guard<std::mutex> g(r->mu);
  r->typ.assign(typ, typ + n);
  for (auto& kv : r->scratch)  // tolerances are baked into captured graphs
    if (kv.second.gexec) { cudaGraphExecDestroy(kv.second.gexec); kv.second.gexec = nullptr; kv.second.gkey.clear(); }
  return 0;
}

}  // extern "C"

namespace {

// Enqueues one advance of the prepared box table on `st` (a captured graph is replayed when the
// box table and dt repeat); the caller holds r->mu.
}  // namespace

namespace pgb_tune {

// Copies cells c = i * stride (i < nsample) of the box table into a single-box arena, one
// component-major block per field: rhoY (ns), rhoY forcing (ns), T, rho h, rho h forcing, FC.
__global__ void gather_sample_kernel(const pgb::BoxDev* boxes, int nbox, int ns, long long nsample, long long stride,
                                     double* arena) {
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < nsample; i += (long long)gridDim.x * blockDim.x) {
    const long long c = i * stride;
    int lo = 0, hi = nbox - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (boxes[mid].cell_offset <= c) lo = mid; else hi = mid - 1;
    }
    const pgb::BoxDev& B = boxes[lo];
    long long r = c - B.cell_offset;
    const int ci = B.lo0 + (int)(r % B.len0);
    r /= B.len0;
    const int cj = B.lo1 + (int)(r % B.len1);
    const int ck = B.lo2 + (int)(r / B.len1);
    auto at = [&](const pgb::ArrDev& a, int n) {
      return a.p[(long long)(ci - a.begin0) + (long long)(cj - a.begin1) * a.jstride + (long long)(ck - a.begin2) * a.kstride +
                 (long long)n * a.nstride];
    };
    for (int k = 0; k < ns; ++k) {
      arena[(size_t)k * nsample + i] = at(B.rY, k) * B.sY_in;
      arena[(size_t)(ns + k) * nsample + i] = at(B.rYsrc, k) * B.sY_in;
    }
    arena[(size_t)(2 * ns) * nsample + i] = at(B.T, 0);
    arena[(size_t)(2 * ns + 1) * nsample + i] = at(B.rE, 0) * B.sE_in;
    arena[(size_t)(2 * ns + 2) * nsample + i] = at(B.rEsrc, 0) * B.sE_in;
    arena[(size_t)(2 * ns + 3) * nsample + i] = 0.0;
  }
}

}  // namespace pgb_tune

namespace {

// gb.autotune: on the first advance, copy a strided sample of the caller's cells (at most
// 32768) into reactor scratch and time one advance of it with every compiled BDF mapping
// (cell per thread with the planner's layout; cell per warp at each compiled warps-per-block
// size whose shared memory fits); keep the fastest for the life of the reactor. The caller's
// arrays are only read. The surrogate (if any) is not part of the timing.
int run_autotune(pgb_reactor* r, const std::vector<pgb::BoxDev>& boxes, long long ncell, double dt, cudaStream_t st) {
  r->tuned = true;
  const MechEntry& m = *r->mech;
  const int ns = m.ns, nf = 2 * ns + 4;
  const long long nsample = std::min<long long>(ncell, 32768);
  const long long stride = std::max<long long>(1, ncell / nsample);
  const size_t arena_bytes = (size_t)nf * nsample * sizeof(double);
  struct Cand { int mapping, wpb; };  // wpb: warps per block (warp mapping), lanes per cell (group)
  std::vector<Cand> cands;
  if (m.bdf_mixed) cands.push_back({0, 0});
  const int per = r->opt.mixed ? m.wsmem_mixed : m.wsmem_fp64;
  for (int i = 0; i < 4 && m.wpb_choice[i] > 0; ++i)
    if (m.wpb_choice[i] * per <= kMaxSmemPerBlock) cands.push_back({1, m.wpb_choice[i]});
  if (m.group_mixed)
    for (int G : {8, 4})
      if ((r->opt.mixed ? m.group_cells_mixed : m.group_cells_fp64)(G) > 0) cands.push_back({2, G});
  if (cands.size() < 2) {
    r->tuning = "single compiled mapping: nothing to tune";
    return 0;
  }
  double* pristine = nullptr;
  double* work = nullptr;
  pgb::BoxDev* d_src = nullptr;
  Scratch sc;
  int rc = 0;
  const Options saved = r->opt;
  SgModel sg_saved = r->sg;
  r->sg.d_net = nullptr;  // time the BDF alone
  auto fail = [&](const char* what) { rc = set_err("autotune: %s", what); };
  do {
    if (cudaMalloc(&pristine, arena_bytes) != cudaSuccess || cudaMalloc(&work, arena_bytes) != cudaSuccess ||
        cudaMalloc(&d_src, boxes.size() * sizeof(pgb::BoxDev)) != cudaSuccess) { fail("out of memory"); break; }
    if (cudaMemcpyAsync(d_src, boxes.data(), boxes.size() * sizeof(pgb::BoxDev), cudaMemcpyHostToDevice, st) != cudaSuccess) {
      fail("box copy"); break;
    }
    pgb_tune::gather_sample_kernel<<<(int)std::min<long long>((nsample + 255) / 256, 1024), 256, 0, st>>>(
        d_src, (int)boxes.size(), ns, nsample, stride, pristine);
    if (cudaGetLastError() != cudaSuccess) { fail("gather launch"); break; }
    if (cudaMalloc(&sc.d_counter, sizeof(unsigned long long)) != cudaSuccess ||
        cudaMalloc(&sc.d_stats, sizeof(pgb::ReactStats)) != cudaSuccess ||
        cudaMalloc(&sc.d_boxes, sizeof(pgb::BoxDev)) != cudaSuccess ||
        cudaMallocHost(&sc.h_boxes, sizeof(pgb::BoxDev)) != cudaSuccess) { fail("out of memory"); break; }
    sc.box_cap = 1;
    pgb::BoxDev& b = *sc.h_boxes;
    std::memset(&b, 0, sizeof(b));
    b.len0 = (int)nsample; b.len1 = 1; b.len2 = 1;
    b.sY_in = b.sE_in = b.sY_out = b.sE_out = 1.0;
    auto field = [&](int f) {
      pgb::ArrDev a;
      std::memset(&a, 0, sizeof(a));
      a.p = work + (size_t)f * nsample;
      a.jstride = nsample; a.kstride = nsample; a.nstride = nsample;
      return a;
    };
    b.rY = field(0); b.rYsrc = field(ns); b.T = field(2 * ns); b.rE = field(2 * ns + 1); b.rEsrc = field(2 * ns + 2);
    b.FC = field(2 * ns + 3);
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess) { fail("events"); break; }
    std::ostringstream rep;
    double best = 1e300;
    Cand pick = cands[0];
    auto name = [](const Cand& c) {
      return c.mapping == 0 ? std::string("thread")
                            : (c.mapping == 1 ? "warp/" : "group/") + std::to_string(c.wpb);
    };
    for (const Cand& c : cands) {
      r->opt.mapping = c.mapping;
      if (c.mapping == 2) r->opt.group = c.wpb; else r->opt.wpb = c.wpb;
      const LaunchPlan pl = plan_launch(r, nsample, r->opt.mixed);
      if (ensure_buf(sc, sc.d_z, sc.z_cap, pl.z_bytes) || ensure_buf(sc, sc.d_lu, sc.lu_cap, pl.lu_bytes)) { rc = -1; break; }
      float ms = 0.f;
      for (int rep_i = 0; rep_i < 2 && !rc; ++rep_i) {  // warm-up launch, then the timed one
        if (cudaMemcpyAsync(work, pristine, arena_bytes, cudaMemcpyDeviceToDevice, st) != cudaSuccess) { fail("copy"); break; }
        cudaEventRecord(e0, st);
        if (enqueue_advance(r, sc, 1, nsample, dt, st)) { rc = -1; break; }
        cudaEventRecord(e1, st);
        if (cudaEventSynchronize(e1) != cudaSuccess) { fail("timed advance failed"); break; }
        cudaEventElapsedTime(&ms, e0, e1);
      }
      if (rc) break;
      rep << name(c) << " " << ms << " ms; ";
      if (ms < best) { best = ms; pick = c; }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) break;
    r->opt = saved;
    r->opt.mapping = pick.mapping;
    if (pick.mapping == 2) r->opt.group = pick.wpb; else r->opt.wpb = pick.wpb;
    rep << "on " << nsample << " sample cells -> " << name(pick);
    r->tuning = rep.str();
  } while (false);
  if (rc) r->opt = saved;
  r->sg = sg_saved;
  cudaStreamSynchronize(st);
  if (pristine) cudaFree(pristine);
  if (work) cudaFree(work);
  if (d_src) cudaFree(d_src);
  free_scratch(sc);
  return rc;
}

int advance_box_table(pgb_reactor* r, const std::vector<pgb::BoxDev>& boxes, long long ncell, double dt_react,
                      cudaStream_t st) {
  const int nbox = (int)boxes.size();
  if (r->opt.autotune && !r->tuned && !r->null_reactor && ncell > 0 && run_autotune(r, boxes, ncell, dt_react, st))
    return -1;
  Scratch* s = nullptr;
  if (ensure_scratch(r, st, std::max(nbox, 1), &s)) return -1;
  if (!r->null_reactor) {
    LaunchPlan pl = plan_launch(r, ncell, r->opt.mixed);
    if (r->opt.mixed && r->opt.retry) {  // the FP64 retry pass shares the global scratch
      const LaunchPlan p64 = plan_launch(r, ncell, false);
      pl.z_bytes = std::max(pl.z_bytes, p64.z_bytes);
      pl.lu_bytes = std::max(pl.lu_bytes, p64.lu_bytes);
      if (ensure_buf(*s, s->d_retry, s->retry_cap, std::max<long long>(ncell, 1) * sizeof(long long))) return -1;
    }
    if (ensure_buf(*s, s->d_z, s->z_cap, pl.z_bytes) || ensure_buf(*s, s->d_lu, s->lu_cap, pl.lu_bytes))
      return -1;
    if (r->sg.d_net) {
      const long long acap = audit_capacity(r, ncell);
      if (ensure_buf(*s, s->d_fallback, s->fallback_cap, std::max<long long>(ncell, 1) * sizeof(long long)) ||
          ensure_buf(*s, s->d_audit, s->audit_cap,
                     std::max<long long>(acap, 1) * (sizeof(long long) + pgb::MAXN * sizeof(double))))
        return -1;
    }
  }
  PGB_CUDA(cudaEventSynchronize(s->done));  // staging buffer may still feed a previous copy
  if (nbox) std::memcpy(s->h_boxes, boxes.data(), nbox * sizeof(pgb::BoxDev));
  s->last_ncell = ncell;
  r->last_stream = st;
  if (r->opt.graph && st != nullptr) {
    if (!(s->gexec && s->gdt == dt_react && same_boxes(s->gkey, boxes.data(), nbox))) {
      if (s->gexec) { cudaGraphExecDestroy(s->gexec); s->gexec = nullptr; }
      cudaGraph_t graph;
      PGB_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
      graph = nullptr;
      const int rc = enqueue_advance(r, *s, nbox, ncell, dt_react, st);
      const cudaError_t ec = cudaStreamEndCapture(st, &graph);
      if (rc || ec != cudaSuccess) {  // the partial graph (if any) is released on every path
        if (graph) cudaGraphDestroy(graph);
        return rc ? rc : set_err("graph capture failed: %s", cudaGetErrorString(ec));
      }
      const cudaError_t ei = cudaGraphInstantiate(&s->gexec, graph, 0);
      cudaGraphDestroy(graph);
      if (ei != cudaSuccess) {
        s->gexec = nullptr;
        return set_err("graph instantiation failed: %s", cudaGetErrorString(ei));
      }
      s->gkey = boxes;
      s->gdt = dt_react;
    }
    PGB_CUDA(cudaGraphLaunch(s->gexec, st));
  } else {
    if (enqueue_advance(r, *s, nbox, ncell, dt_react, st)) return -1;
  }
  PGB_CUDA(cudaEventRecord(s->done, st));
  return 0;
}

}  // namespace

extern "C" {

int pgb_reactor_react_boxes(pgb_reactor* r, const pgb_box_view* views, int nbox, double dt_react,
                            double time, void* stream) {
  (void)time;
  if (!r) return set_err("null reactor");
  if (nbox < 0 || (nbox > 0 && !views)) return set_err("bad box list");
  if (!(dt_react > 0.0)) return set_err("dt_react must be > 0");
  std::lock_guard<std::mutex> g(r->mu);
  std::vector<pgb::BoxDev> boxes;
  long long ncell = 0;
  if (build_boxes(views, nbox, r->mech->ns, boxes, ncell)) return -1;
  return advance_box_table(r, boxes, ncell, dt_react, static_cast<cudaStream_t>(stream));
}

int pgb_advance_chemistry(pgb_reactor* r, const pgb_chem_view* views, int nbox, double dt, void* stream) {
  if (!r) return set_err("null reactor");
  if (nbox < 0 || (nbox > 0 && !views)) return set_err("bad box list");
  if (!(dt > 0.0)) return set_err("dt must be > 0");
  if (r->sg.d_net) return set_err("advance_chemistry: the surrogate path takes CGS arrays (react_boxes)");
  std::vector<pgb_box_view> bv(nbox);
  for (int b = 0; b < nbox; ++b) {
    const pgb_chem_view& c = views[b];
    pgb_box_view& v = bv[b];
    std::memset(&v, 0, sizeof(v));
    v.box = c.box;
    v.rY = c.rhoY; v.rY_src = c.rhoY_src; v.T = c.T; v.rEner = c.rhoH; v.rEner_src = c.rhoH_src;
    v.FC = c.FC; v.mask = c.mask;
    if (c.I_R.p && check_arr(c.I_R, c.box, r->mech->ns, "I_R", b)) return -1;
  }
  std::lock_guard<std::mutex> g(r->mu);
  std::vector<pgb::BoxDev> boxes;
  long long ncell = 0;
  if (build_boxes(bv.data(), nbox, r->mech->ns, boxes, ncell)) return -1;
  for (int b = 0; b < nbox; ++b) {  // MKS <-> CGS as advance_chemistry does (Source/PeleLM.cpp:5736-5771)
    boxes[b].sY_in = 1.0e-3;
    boxes[b].sE_in = 10.0;
    boxes[b].sY_out = 1.0e3;
    boxes[b].sE_out = 0.1;
    if (views[b].I_R.p) boxes[b].IR = arr_dev(views[b].I_R);
  }
  return advance_box_table(r, boxes, ncell, dt, static_cast<cudaStream_t>(stream));
}

int pgb_reactor_tuning(pgb_reactor* r, char* buf, size_t n) {
  if (!r) return set_err("null reactor");
  std::lock_guard<std::mutex> g(r->mu);
  if (buf && n) {
    std::strncpy(buf, r->tuning.c_str(), n - 1);
    buf[n - 1] = 0;
  }
  return (int)r->tuning.size();
}

int pgb_reactor_get_stats(pgb_reactor* r, pgb_stats* out) {
  if (!r || !out) return set_err("null argument");
  std::lock_guard<std::mutex> g(r->mu);
  auto it = r->scratch.find(r->last_stream);
  if (it == r->scratch.end()) return set_err("no advance has run yet");
  Scratch& s = it->second;
  pgb::ReactStats h;
  PGB_CUDA(cudaEventSynchronize(s.done));
  PGB_CUDA(cudaMemcpy(&h, s.d_stats, sizeof(h), cudaMemcpyDeviceToHost));
  out->ncell = (unsigned long long)s.last_ncell;
  out->nst = h.nst; out->nfe = h.nfe; out->nje = h.nje; out->netf = h.netf; out->ncfn = h.ncfn;
  out->nfail = h.nfail; out->max_nst = h.max_nst;
  for (int i = 0; i < 16; ++i) out->hist[i] = h.hist[i];
  out->nretry = h.nretry;
  return 0;
}

int pgb_reactor_get_surrogate_stats(pgb_reactor* r, pgb_surrogate_stats* out) {
  if (!r || !out) return set_err("null argument");
  if (!r->sg.d_net) return set_err("reactor has no surrogate (gb.surrogate)");
  std::lock_guard<std::mutex> g(r->mu);
  auto it = r->scratch.find(r->last_stream);
  if (it == r->scratch.end()) return set_err("no advance has run yet");
  Scratch& s = it->second;
  pgb::SurrogateStats h;
  PGB_CUDA(cudaEventSynchronize(s.done));
  PGB_CUDA(cudaMemcpy(&h, s.d_sg_stats, sizeof(h), cudaMemcpyDeviceToHost));
  out->ncell = h.ncell; out->accept = h.accept; out->fallback = h.fallback;
  out->ood = h.ood; out->mis = h.mis; out->cons = h.cons; out->ens = h.ens; out->neg = h.neg;
  out->audit = h.audit; out->audit_bad = h.audit_bad;
  std::memcpy(&out->audit_max_dT, &h.audit_max_dT, sizeof(double));
  std::memcpy(&out->audit_max_dY, &h.audit_max_dY, sizeof(double));
  return 0;
}

int pgb_reactor_surrogate_raw(pgb_reactor* r, const pgb_box_view* views, int nbox, float* out,
                              float* in_rows, void* stream) {
  if (!r || !views || !out || nbox < 1) return set_err("surrogate_raw: null argument");
  if (!r->sg.d_net) return set_err("reactor has no surrogate (gb.surrogate)");
  std::vector<pgb::BoxDev> boxes;
  long long ncell = 0;
  if (build_boxes(views, nbox, r->mech->ns, boxes, ncell)) return -1;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  pgb::BoxDev* d = nullptr;
  PGB_CUDA(cudaMalloc(&d, nbox * sizeof(pgb::BoxDev)));
  int rc = 0;
  if (cudaMemcpyAsync(d, boxes.data(), nbox * sizeof(pgb::BoxDev), cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = set_err("surrogate_raw: box table copy failed");
  unsigned long long* seed = nullptr;
  if (!rc && cudaMalloc(&seed, sizeof(unsigned long long)) != cudaSuccess) rc = set_err("surrogate_raw: no memory");
  if (!rc && cudaMemsetAsync(seed, 0, sizeof(unsigned long long), st) != cudaSuccess) rc = set_err("surrogate_raw: memset");
  if (!rc) {
    pgb::SurrogateParams sp;
    std::memset(&sp, 0, sizeof(sp));
    sp.boxes = d;
    sp.nbox = nbox;
    sp.ncell = ncell;
    sp.net = r->sg.d_net;
    sp.seed_dev = seed;
    sp.raw_out = out;
    sp.raw_in = in_rows;
    const long long ntiles = (ncell + pgb::SG_TILE - 1) / pgb::SG_TILE;
    rc = r->mech->sg_fn(sp, st, (int)std::min<long long>(ntiles, r->nsm));
  }
  if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = set_err("surrogate_raw: kernel failed");
  cudaFree(seed);
  cudaFree(d);
  return rc;
}

int pgb_surrogate_features(const char* mechanism, const pgb_box_view* views, int nbox, float* out,
                           void* stream) {
  const MechEntry* m = find_mech(mechanism);
  if (!m) return set_err("unknown mechanism '%s'", mechanism ? mechanism : "(null)");
  if (!m->sg_feat_fn) return set_err("no surrogate features are compiled for mechanism '%s'", m->name);
  if (nbox < 1 || !views || !out) return set_err("surrogate_features: need boxes and an output array");
  std::vector<pgb::BoxDev> boxes;
  long long ncell = 0;
  if (build_boxes(views, nbox, m->ns, boxes, ncell)) return -1;
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  pgb::BoxDev* d = nullptr;
  PGB_CUDA(cudaMalloc(&d, nbox * sizeof(pgb::BoxDev)));
  int rc = 0;
  if (cudaMemcpyAsync(d, boxes.data(), nbox * sizeof(pgb::BoxDev), cudaMemcpyHostToDevice, st) != cudaSuccess)
    rc = set_err("surrogate_features: box table copy failed");
  if (!rc) rc = m->sg_feat_fn(d, nbox, ncell, out, st);
  if (cudaStreamSynchronize(st) != cudaSuccess && !rc) rc = set_err("surrogate_features: kernel failed");
  cudaFree(d);
  return rc;
}

int pgb_reactor_react(pgb_reactor* r, const pgb_box_view* view, double* dt_react, double* time,
                      void* stream) {
  if (!r || !view || !dt_react || !time) return set_err("null argument");
  if (pgb_reactor_react_boxes(r, view, 1, *dt_react, *time, stream)) return -1;
  pgb_stats st;
  if (pgb_reactor_get_stats(r, &st)) return -1;
  return (int)st.nfail;
}

void pgb_reactor_close(pgb_reactor* r) {
  if (!r) return;
  {
    std::lock_guard<std::mutex> g(r->mu);
    for (auto& kv : r->scratch) {
      if (kv.second.done) cudaEventSynchronize(kv.second.done);
      free_scratch(kv.second);
    }
    sg_free(r->sg);
  }
  delete r;
}

int pgb_reaction_rates(const char* mechanism, const pgb_box_view* view, const pgb_array4* out,
                       void* stream) {
  const MechEntry* m = find_mech(mechanism);
  if (!m) return set_err("unknown mechanism '%s'", mechanism ? mechanism : "(null)");
  if (!view || !out) return set_err("null argument");
  if (!m->rates_fn) return set_err("pointwise rates are not compiled for mechanism '%s'", m->name);
  return m->rates_fn(view, out, static_cast<cudaStream_t>(stream));
}

int pgb_heat_release(const char* mechanism, const pgb_box* box, const pgb_array4* T,
                     const pgb_array4* rhoYdot, const pgb_array4* hr, void* stream) {
  const MechEntry* m = find_mech(mechanism);
  if (!m) return set_err("unknown mechanism '%s'", mechanism ? mechanism : "(null)");
  if (!box || !T || !rhoYdot || !hr) return set_err("null argument");
  for (int d = 0; d < 3; ++d)
    if (box->hi[d] < box->lo[d]) return set_err("heat_release: empty box");
  return m->hr_fn(box, T, rhoYdot, hr, static_cast<cudaStream_t>(stream));
}

int pgb_newton_matrix(const char* mechanism, int mapping, long long ncell, const double* y,
                      const double* F, const double* Fh, double gamma, const double* b, int fp64,
                      double* J, double* x, void* stream) {
  const MechEntry* m = find_mech(mechanism);
  if (!m) return set_err("unknown mechanism '%s'", mechanism ? mechanism : "(null)");
  if (ncell < 0) return set_err("newton_matrix: ncell must be >= 0");
  if (ncell > 0 && (!y || !F || !Fh || !b || !J || !x)) return set_err("null argument");
  if (!m->newton_fn) return set_err("the Newton matrix diagnostic is not compiled for mechanism '%s'", m->name);
  pgb::NewtonMatrixParams p;
  p.ncell = ncell; p.y = y; p.F = F; p.Fh = Fh; p.b = b; p.gamma = gamma; p.J = J; p.x = x;
  return m->newton_fn(p, mapping, fp64, static_cast<cudaStream_t>(stream));
}

int pgb_rhoh_to_temp(const char* mechanism, const pgb_box_view* view, double tmin, double tmax,
                     void* stream) {
  const MechEntry* m = find_mech(mechanism);
  if (!m) return set_err("unknown mechanism '%s'", mechanism ? mechanism : "(null)");
  if (!view) return set_err("null argument");
  if (!(tmin > 0.0 && tmax > tmin)) return set_err("need 0 < tmin < tmax");
  return m->h2t_fn(view, tmin, tmax, static_cast<cudaStream_t>(stream));
}

}  // extern "C"

namespace {

const MechEntry* const kMechs[] = {PGB_MECH_LIST};

const MechEntry* find_mech(const char* name) {
  if (!name) return nullptr;
  for (const MechEntry* m : kMechs)
    if (std::strcmp(m->name, name) == 0) return m;
  return nullptr;
}

}  // namespace

const pgb_host::MechEntry* pgb_host::find_mech_entry(const char* name) { return find_mech(name); }
