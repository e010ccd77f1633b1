// Host-side handle of a loaded surrogate (surrogate_io.cu).
#ifndef PGB_SURROGATE_HOST_H
#define PGB_SURROGATE_HOST_H

#include <cmath>

#include "reactor_registry.cuh"
#include "surrogate_kernel.cuh"

namespace pgb_host {

// Runtime overrides of the thresholds stored in the file (NaN / 0 = keep the file's value).
struct SgOverrides {
  double ood_margin = NAN, mis = NAN, cons = NAN, disT = NAN, disY = NAN, neg = NAN;
  double tol_T = NAN, tol_Y = NAN, audit_frac = NAN;
  int models = 0;  // use only the first `models` ensemble members
};

struct SgModel {
  pgb::SurrogateNet* d_net = nullptr;
  void* d_weights = nullptr;
  double audit_frac = 0.0;
  int nmodel = 0;
};

int sg_load(const char* path, const char* mech_name, int ns, const SgOverrides& ov, SgModel& out);
void sg_free(SgModel& m);

}  // namespace pgb_host

#endif  // PGB_SURROGATE_HOST_H
