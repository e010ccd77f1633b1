"""The header-only C++ binding for AMReX/PeleLM callers (include/pelelm_gb300_amrex.H) compiles
against the AMReX names it uses and a ReactorBase with the interface PeleLM calls
(Source/PeleLM.cpp:706-709, :1513, :5752-5757, :930), with and without AMREX_USE_GPU, links the
library and forwards: argument errors come back through amrex::Abort with the library's message,
and Array4/Box views convert field by field. The AMReX and ReactorBase stand-ins below declare
only those names (no GPU needed)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

STUBS = {
    "AMReX.H": """#pragma once
#include <stdexcept>
#include <string>
namespace amrex {
using Real = double;
using Long = long long;
[[noreturn]] inline void Abort(const std::string& m) { throw std::runtime_error(m); }
}
""",
    "AMReX_Array4.H": """#pragma once
#include "AMReX.H"
namespace amrex {
struct Dim3 { int x, y, z; };
template <class T> struct Array4 {
  T* p = nullptr;
  Long jstride = 0, kstride = 0, nstride = 0;
  Dim3 begin{1, 1, 1}, end{0, 0, 0};
  int ncomp = 0;
};
}
""",
    "AMReX_Box.H": """#pragma once
namespace amrex {
struct Box {
  int lo[3], hi[3];
  int smallEnd(int d) const { return lo[d]; }
  int bigEnd(int d) const { return hi[d]; }
};
}
""",
    "AMReX_Gpu.H": """#pragma once
namespace amrex { using gpuStream_t = struct stand_in_stream*; }
""",
}

MAIN = r"""
#include <cstdio>
#include <cstring>
#include <memory>
#include <vector>
#include <AMReX.H>
#include <AMReX_Array4.H>
#include <AMReX_Box.H>
#ifdef AMREX_USE_GPU
#include <AMReX_Gpu.H>
#endif
struct ReactorBase {
  virtual ~ReactorBase() = default;
  virtual void init(int reactor_type, int ncells) = 0;
  virtual void set_typ_vals_ode(const std::vector<amrex::Real>& typ) = 0;
  virtual int react(const amrex::Box& box, amrex::Array4<amrex::Real> const& rY_in,
                    amrex::Array4<amrex::Real> const& rY_src_in, amrex::Array4<amrex::Real> const& T_in,
                    amrex::Array4<amrex::Real> const& rEner_in, amrex::Array4<amrex::Real> const& rEner_src_in,
                    amrex::Array4<amrex::Real> const& FC_in, amrex::Array4<int> const& mask,
                    amrex::Real& dt_react, amrex::Real& time
#ifdef AMREX_USE_GPU
                    , amrex::gpuStream_t stream
#endif
                    ) = 0;
  virtual void close() = 0;
};
#include "pelelm_gb300_amrex.H"

int main() {
  std::unique_ptr<ReactorBase> r = std::make_unique<pgb::ReactorGB<ReactorBase>>("drm19_syn", "ode.rtol=abc");
  try { r->init(2, 1); return 1; } catch (const std::runtime_error& e) {
    if (!std::strstr(e.what(), "bad value")) return 2;
  }
  r->close();
  pgb::ReactorGB<ReactorBase> g("no_such_mechanism", "");
  try { g.init(2, 1); return 3; } catch (const std::runtime_error& e) {
    if (!std::strstr(e.what(), "unknown mechanism")) return 4;
  }
  static double buf[2 * 3 * 4 * 5];
  amrex::Array4<amrex::Real> a;
  a.p = buf; a.jstride = 5; a.kstride = 20; a.nstride = 60;
  a.begin = {-1, 2, 3}; a.end = {4, 6, 6}; a.ncomp = 2;
  amrex::Array4<int> m;
  const amrex::Box bx{{-1, 2, 3}, {3, 5, 5}};
  const pgb_box_view v = pgb::box_view(bx, a, a, a, a, a, a, m);
  if (v.rY.p != buf || v.T.jstride != 5 || v.FC.kstride != 20 || v.rEner.nstride != 60) return 5;
  if (v.rY.begin[0] != -1 || v.rY.begin[2] != 3 || v.rY.end[1] != 6 || v.rY.ncomp != 2) return 6;
  if (v.mask.p != nullptr || v.box.lo[0] != -1 || v.box.hi[2] != 5) return 7;
  std::printf("ok\n");
  return 0;
}
"""


@pytest.mark.parametrize("gpu", [False, True])
def test_amrex_binding_compiles_and_forwards(native_lib, tmp_path, gpu):
    if not shutil.which("g++"):
        pytest.skip("g++ not installed")
    from pelelm_gb300._build import LIB
    stub = tmp_path / "stub"
    stub.mkdir()
    for name, text in STUBS.items():
        (stub / name).write_text(text)
    src = tmp_path / "main.cpp"
    src.write_text(MAIN)
    exe = tmp_path / "binding_check"
    libdir = os.path.dirname(LIB)
    cmd = ["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-I", str(stub), "-I", os.path.join(ROOT, "include"),
           str(src), "-L", libdir, "-lpelelm_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)]
    if gpu:
        cmd.insert(1, "-DAMREX_USE_GPU")
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0 and out.stdout.strip() == "ok", (out.returncode, out.stdout, out.stderr)
