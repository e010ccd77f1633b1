/* Header-only C++ binding of the pelelm_gb300 C ABI for AMReX/PeleLM callers.
 *
 * pgb::ReactorGB<Base> implements the PelePhysics reactor interface that PeleLM holds in
 * `static std::unique_ptr<pele::physics::reactions::ReactorBase> m_reactor`
 * (Source/PeleLM.H:673-674) and calls as create/init (Source/PeleLM.cpp:706-709),
 * set_typ_vals_ode (:1513), react (:5752-5757) and close (:930), by forwarding each call to
 * pgb_reactor_* (pelelm_gb300.h). Base is the reference's ReactorBase, so this header compiles
 * without PelePhysics:
 *
 *     #include <PelePhysics reactor headers>
 *     #include <pelelm_gb300_amrex.H>
 *     using ReactorGB = pgb::ReactorGB<pele::physics::reactions::ReactorBase>;
 *     m_reactor = std::make_unique<ReactorGB>("drm19_syn", "ode.rtol=1e-6 ode.atol=1e-10");
 *
 * Needs AMReX (Array4, Box, Real, Abort; gpuStream_t when AMREX_USE_GPU is defined). Errors
 * from the library end in amrex::Abort with its message; react returns the number of failed
 * cells, as the reference's does. Any further pure virtual member that the PelePhysics version
 * at hand declares in ReactorBase is added to a subclass by the integrator.
 */
#ifndef PELELM_GB300_AMREX_H
#define PELELM_GB300_AMREX_H

#include <AMReX.H>
#include <AMReX_Array4.H>
#include <AMReX_Box.H>
#ifdef AMREX_USE_GPU
#include <AMReX_Gpu.H>
#endif

#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include "pelelm_gb300.h"

namespace pgb {

/* pgb_array4 view of an amrex::Array4 (same pointer, strides and index bounds). */
template <class T>
inline pgb_array4 to_pgb(const amrex::Array4<T>& a) {
  pgb_array4 v{};
  v.p = const_cast<void*>(static_cast<const void*>(a.p));
  v.jstride = a.jstride;
  v.kstride = a.kstride;
  v.nstride = a.nstride;
  v.begin[0] = a.begin.x;
  v.begin[1] = a.begin.y;
  v.begin[2] = a.begin.z;
  v.end[0] = a.end.x;
  v.end[1] = a.end.y;
  v.end[2] = a.end.z;
  v.ncomp = a.ncomp;
  return v;
}

inline pgb_box to_pgb(const amrex::Box& bx) {
  pgb_box b{};
  for (int d = 0; d < 3; ++d) {
    b.lo[d] = bx.smallEnd(d);
    b.hi[d] = bx.bigEnd(d);
  }
  return b;
}

inline std::string last_error() {
  char buf[1024];
  pgb_last_error(buf, sizeof buf);
  return std::string(buf);
}

/* The arguments of one react call as a box view (the fields of pgb_box_view). */
inline pgb_box_view box_view(const amrex::Box& bx, amrex::Array4<amrex::Real> const& rY,
                             amrex::Array4<amrex::Real> const& rY_src,
                             amrex::Array4<amrex::Real> const& T,
                             amrex::Array4<amrex::Real> const& rEner,
                             amrex::Array4<amrex::Real> const& rEner_src,
                             amrex::Array4<amrex::Real> const& FC, amrex::Array4<int> const& mask) {
  pgb_box_view v{};
  v.box = to_pgb(bx);
  v.rY = to_pgb(rY);
  v.rY_src = to_pgb(rY_src);
  v.T = to_pgb(T);
  v.rEner = to_pgb(rEner);
  v.rEner_src = to_pgb(rEner_src);
  v.FC = to_pgb(FC);
  v.mask = to_pgb(mask);
  return v;
}

template <class Base>
class ReactorGB : public Base {
  static_assert(std::is_same<amrex::Real, double>::value, "pelelm_gb300 integrates in double");

 public:
  /* mechanism: one compiled into the library (pgb_mechanism_info); options: the runtime keys of
   * pgb_reactor_create (the reference's ode.* / cvode.* names plus gb.*). */
  ReactorGB(std::string mechanism, std::string options)
      : mech_(std::move(mechanism)), opts_(std::move(options)) {}
  ~ReactorGB() override { release(); }

  void init(int reactor_type, int /*ncells*/) override {
    release();
    r_ = pgb_reactor_create("ReactorCvode", mech_.c_str(), reactor_type, opts_.c_str());
    if (!r_) amrex::Abort("pelelm_gb300: " + last_error());
  }

  void set_typ_vals_ode(const std::vector<amrex::Real>& typ) override {
    if (pgb_reactor_set_typ_vals_ode(r_, typ.data(), static_cast<int>(typ.size())) < 0)
      amrex::Abort("pelelm_gb300: " + last_error());
  }

  int react(const amrex::Box& bx, amrex::Array4<amrex::Real> const& rY_in,
            amrex::Array4<amrex::Real> const& rY_src_in, amrex::Array4<amrex::Real> const& T_in,
            amrex::Array4<amrex::Real> const& rEner_in,
            amrex::Array4<amrex::Real> const& rEner_src_in, amrex::Array4<amrex::Real> const& FC_in,
            amrex::Array4<int> const& mask, amrex::Real& dt_react, amrex::Real& time
#ifdef AMREX_USE_GPU
            , amrex::gpuStream_t stream
#endif
            ) override {
#ifdef AMREX_USE_GPU
    void* s = reinterpret_cast<void*>(stream);
#else
    void* s = nullptr;
#endif
    const pgb_box_view v = box_view(bx, rY_in, rY_src_in, T_in, rEner_in, rEner_src_in, FC_in, mask);
    const int nfail = pgb_reactor_react(r_, &v, &dt_react, &time, s);
    if (nfail < 0) amrex::Abort("pelelm_gb300: " + last_error());
    return nfail;
  }

  void close() override { release(); }

  /* Every box of a level (or of all levels) in one persistent launch, stream ordered
   * (pgb_reactor_react_boxes): build the views with box_view() inside the MFIter loop and call
   * this once after it instead of react() per box. Returns 0, or aborts with the message. */
  int react_boxes(const std::vector<pgb_box_view>& views, amrex::Real dt_react, void* stream) {
    const int rc = pgb_reactor_react_boxes(r_, views.data(), static_cast<int>(views.size()), dt_react,
                                           0.0, stream);
    if (rc < 0) amrex::Abort("pelelm_gb300: " + last_error());
    return rc;
  }

  /* Counters of the last advance (steps, RHS evaluations, Jacobians, failures, retries). */
  pgb_stats stats() const {
    pgb_stats s{};
    if (pgb_reactor_get_stats(r_, &s) < 0) amrex::Abort("pelelm_gb300: " + last_error());
    return s;
  }

 private:
  void release() {
    if (r_) pgb_reactor_close(r_);
    r_ = nullptr;
  }
  std::string mech_, opts_;
  pgb_reactor* r_ = nullptr;
};

}  // namespace pgb

#endif  // PELELM_GB300_AMREX_H
