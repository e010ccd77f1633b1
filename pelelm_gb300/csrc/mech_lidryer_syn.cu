// Kernels of the lidryer_syn mechanism (persistent BDF in mixed and FP64 precision, pointwise
// rates / T(h) / null reactor) and its registry entry.
#include "gen/mech_lidryer_syn.cuh"
#include "reactor_registry.cuh"

namespace pgb_host {
extern const MechEntry kEntry_lidryer_syn = PGB_MECH_ENTRY(pgb::Mech_lidryer_syn);
}  // namespace pgb_host
