"""The product library loads and exports the C ABI declared in include/pelelm_gb300.h; argument
errors come back as -1 / NULL with a message (no GPU needed for these)."""
import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "pelelm_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pgb_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_reactor_interface():
    syms = declared_symbols()
    for s in ("pgb_reactor_create", "pgb_reactor_set_typ_vals_ode", "pgb_reactor_react",
              "pgb_reactor_react_boxes", "pgb_reactor_close", "pgb_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol(native_lib):
    for s in declared_symbols():
        assert hasattr(native_lib, s), f"{s} declared in include/pelelm_gb300.h but not exported"


def test_binding_covers_every_declared_symbol():
    from pelelm_gb300 import _lib
    assert set(declared_symbols()) <= set(_lib.EXPORTS)


def test_version_and_mechanisms(native_lib):
    from pelelm_gb300.reactor import mechanism_info
    assert native_lib.pgb_version() == 1
    assert mechanism_info("lidryer_syn") == (9, 21)
    assert mechanism_info("drm19_syn") == (21, 84)
    with pytest.raises(RuntimeError, match="unknown mechanism"):
        mechanism_info("no_such_mechanism")


@pytest.mark.parametrize("name,mech,rtype,opts,msg", [
    ("ReactorRK64", "lidryer_syn", 2, "", "not provided"),
    ("ReactorFoo", "lidryer_syn", 2, "", "unknown reactor"),
    ("ReactorCvode", "lidryer_syn", 1, "", "reactor_type"),
    ("ReactorCvode", "nope", 2, "", "unknown mechanism"),
    ("ReactorCvode", "lidryer_syn", 2, "ode.rtol=abc", "bad value"),
    ("ReactorCvode", "lidryer_syn", 2, "cvode.max_order=7", "max_order"),
    ("ReactorCvode", "lidryer_syn", 2, "cvode.solve_type=sparse_direct", "not provided"),
    ("ReactorCvode", "lidryer_syn", 2, "gb.precision=fp16", "gb.precision"),
    ("ReactorCvode", "lidryer_syn", 2, "foo.bar=1", "unknown option"),
    ("ReactorCvode", "lidryer_syn", 2, "gb.retry=yes", "bad value"),
])
def test_create_rejects_bad_arguments(native_lib, name, mech, rtype, opts, msg):
    from pelelm_gb300 import _lib
    h = native_lib.pgb_reactor_create(name.encode(), mech.encode(), rtype, opts.encode())
    assert not h
    assert msg in _lib.last_error()


@pytest.mark.parametrize("solve_type", ["GMRES", "precGMRES", "dense", "denseAJ_direct"])
def test_options_of_the_reference_decks_are_accepted(native_lib, solve_type):
    """The option strings of the reference's input decks pass the option parser, including the
    GPU deck's matrix-free key (Exec/RegTests/FlameSheet/inputs.3d-regt_GPU:85-89), which runs
    the dense direct Newton solve. Without a GPU, create() then stops at the device query."""
    from pelelm_gb300 import _lib
    opts = (f"peleLM.use_typ_vals_chem=1 ode.rtol=1.0e-6 ode.atol=1.0e-5 "
            f"cvode.solve_type={solve_type} cvode.max_order=4")
    h = native_lib.pgb_reactor_create(b"ReactorCvode", b"drm19_syn", 2, opts.encode())
    if h:
        native_lib.pgb_reactor_close(h)
    else:
        err = _lib.last_error()
        assert "solve_type" not in err and "option" not in err, err


def test_python_factory_mirrors_reference_names():
    from pelelm_gb300.reactor import ReactorBase
    with pytest.raises(ValueError):
        ReactorBase.create("ReactorArkode")
    r = ReactorBase.create("ReactorCvode", "lidryer_syn", "ode.rtol=1e-6")
    assert (r.ns, r.nr) == (9, 21)


C_PROGRAM = r"""
#include "pelelm_gb300.h"
#include <stdio.h>
#include <string.h>
int main(void) {
  int ns = 0, nr = 0;
  char buf[512];
  pgb_stats st;
  pgb_box_view v;
  pgb_chem_view cv;
  pgb_reactor* r;
  memset(&st, 0, sizeof st);
  memset(&v, 0, sizeof v);
  memset(&cv, 0, sizeof cv);
  if (pgb_version() != PGB_ABI_VERSION) return 1;
  if (pgb_mechanism_info("drm19_syn", &ns, &nr) != 0 || ns != 21 || nr != 84) return 2;
  r = pgb_reactor_create("ReactorRK64", "drm19_syn", 2, "");
  if (r) return 3;
  pgb_last_error(buf, sizeof buf);
  if (!strstr(buf, "not provided")) return 4;
  printf("%d %d %s\n", ns, nr, buf);
  return 0;
}
"""


@pytest.mark.parametrize("compiler,std", [("gcc", "-std=c99"), ("g++", "-std=c++17")])
def test_header_compiles_links_and_calls_from_c(native_lib, tmp_path, compiler, std):
    """The header is plain C (and C++): a program written against it alone compiles with
    warnings as errors, links the library and gets answers and error messages (no GPU call)."""
    import shutil
    import subprocess
    if not shutil.which(compiler):
        pytest.skip(f"{compiler} not installed")
    from pelelm_gb300._build import LIB
    src = tmp_path / ("abi_check.c" if compiler == "gcc" else "abi_check.cpp")
    src.write_text(C_PROGRAM)
    exe = tmp_path / "abi_check"
    libdir = os.path.dirname(LIB)
    subprocess.run([compiler, std, "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
                    str(src), "-L", libdir, "-lpelelm_gb300", f"-Wl,-rpath,{libdir}", "-o", str(exe)],
                   check=True, capture_output=True, text=True)
    out = subprocess.run([str(exe)], capture_output=True, text=True)
    assert out.returncode == 0, (out.returncode, out.stdout, out.stderr)
    assert out.stdout.startswith("21 84 ")
