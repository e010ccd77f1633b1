// Kernels of the drm19_syn mechanism (persistent BDF in mixed and FP64 precision: cell per
// thread, per group of lanes and per warp; pointwise rates / T(h) / null reactor) and its
// registry entry.
#include "gen/mech_drm19_syn.cuh"
#include "reactor_registry.cuh"

namespace pgb_host {
extern const MechEntry kEntry_drm19_syn = PGB_MECH_ENTRY_GROUP(pgb::Mech_drm19_syn);
}  // namespace pgb_host
