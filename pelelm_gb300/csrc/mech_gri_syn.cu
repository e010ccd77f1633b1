// Kernels of the gri_syn mechanism (53 species, 325 reactions): the warp-per-cell persistent BDF
// in mixed and FP64 precision, ReactorNull and T(h, Y), and its registry entry. One cell per
// thread does not fit this size (N = 54: the history, Jacobian and LU of one cell take ~15 KB).
#include "gen/mech_gri_syn.cuh"
#include "reactor_registry.cuh"

namespace pgb_host {
extern const MechEntry kEntry_gri_syn = PGB_MECH_ENTRY_WARP(pgb::Mech_gri_syn);
}  // namespace pgb_host
