// Device-side descriptors shared by the reactor kernels and the host driver.
#ifndef PGB_REACTOR_TYPES_CUH
#define PGB_REACTOR_TYPES_CUH

#include <stdint.h>

namespace pgb {

constexpr int QMAX = 5;     // highest BDF order supported (cvode.max_order <= 5)
constexpr int MAXN = 64;    // largest ODE size (species + 1) any built mechanism uses

// One Array4-like view: element (i,j,k,n) lives at
// p[(i-begin0) + (j-begin1)*jstride + (k-begin2)*kstride + n*nstride].
struct ArrDev {
  double* p;
  long long jstride, kstride, nstride;
  int begin0, begin1, begin2;
};

struct MaskDev {
  const int* p;
  long long jstride, kstride;
  int begin0, begin1, begin2;
};

// One box of cells; cells are numbered i fastest, then j, then k, starting at
// cell_offset within the flat cell index space of one launch.
struct BoxDev {
  int lo0, lo1, lo2;
  int len0, len1, len2;
  long long cell_offset;
  ArrDev rY, rYsrc, T, rE, rEsrc, FC;
  MaskDev mask;  // p may be null: all cells active
  // Units of the caller's arrays: rhoY and its forcing are multiplied by sY_in and rho h and
  // its forcing by sE_in when a cell is loaded, results by sY_out / sE_out when it is written
  // (1 for CGS arrays; 1e-3, 10 / 1e3, 0.1 for PeleLM's MKS state, Source/PeleLM.cpp:5736-5771).
  double sY_in, sE_in, sY_out, sE_out;
  ArrDev IR;  // p may be null; else I_R = -(rhoY_old - rhoY_new) / dt - F_rhoY in the caller's units
};

// Per-launch counters (device scratch, zeroed before each launch).
struct ReactStats {
  unsigned long long nst, nfe, nje, netf, ncfn, nfail;
  unsigned long long max_nst;
  unsigned long long hist[16];  // steps per cell, bins [2^b, 2^(b+1))
  unsigned long long nretry;    // cells handed to the retry list (their work is in nst/nfe/...)
};

struct ReactParams {
  const BoxDev* boxes;
  int nbox;
  long long ncell;
  double dt;
  double rtol;
  double atol[MAXN];
  int max_order;
  int max_steps;
  unsigned long long* next_cell;  // work queue head (device scratch)
  ReactStats* stats;              // device scratch
  void* lu_scratch;               // per-thread Jacobian/LU slices in global memory, or null
  void* z_scratch;                // per-thread Nordsieck histories in global memory, or null
  // Optional indirection (both null for a plain advance): queue entry c < *ncell_dev advances
  // flat cell cell_list[c]. Lets a producer kernel on the same stream hand over a cell subset
  // (the surrogate's fallback cells) without a host round trip.
  const long long* cell_list;
  const unsigned long long* ncell_dev;
  // Optional retry list (null: a failed cell writes its state at failure and its -status to
  // FC): a cell whose integration fails appends its flat index here and leaves every caller
  // array as it found it, so a second pass (FP64 after mixed precision) can start it over.
  long long* retry_list;
  unsigned long long* retry_count;
};

}  // namespace pgb

#endif  // PGB_REACTOR_TYPES_CUH
