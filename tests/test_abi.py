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
    ("ReactorCvode", "lidryer_syn", 2, "cvode.solve_type=GMRES", "not provided"),
    ("ReactorCvode", "lidryer_syn", 2, "gb.precision=fp16", "gb.precision"),
    ("ReactorCvode", "lidryer_syn", 2, "foo.bar=1", "unknown option"),
])
def test_create_rejects_bad_arguments(native_lib, name, mech, rtype, opts, msg):
    from pelelm_gb300 import _lib
    h = native_lib.pgb_reactor_create(name.encode(), mech.encode(), rtype, opts.encode())
    assert not h
    assert msg in _lib.last_error()


def test_python_factory_mirrors_reference_names():
    from pelelm_gb300.reactor import ReactorBase
    with pytest.raises(ValueError):
        ReactorBase.create("ReactorArkode")
    r = ReactorBase.create("ReactorCvode", "lidryer_syn", "ode.rtol=1e-6")
    assert (r.ns, r.nr) == (9, 21)
