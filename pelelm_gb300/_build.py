"""Build recipe for the in-tree native library (sm_103a only) and the CPU oracle.

nvcc compiles each translation unit for ``-gencode arch=compute_103a,code=sm_103a`` in
parallel, then links one shared library ``pelelm_gb300/libpelelm_gb300.so`` (C ABI in
``include/pelelm_gb300.h``). Generated mechanism headers are refreshed from the mechanism
JSON files first.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIB = os.path.join(PKG, "libpelelm_gb300.so")
BUILD = os.path.join(PKG, "_build")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-std=c++17", "-O3", "-lineinfo", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
           "-Xcompiler", "-O2"]
# host and shared units; each mechanism adds a generated csrc/gen/unit_<name>.cu
UNITS = ["reactor.cu", "peak.cu", "noalloc.cu", "partition.cpp", "mlp.cu", "surrogate_io.cu"]
DATA = os.path.join(PKG, "data")


def mechanism_names() -> list:
    """Every mechanism description in pelelm_gb300/data (<name>.json holding species and
    reactions): the three built-in synthetic ones first, then others (e.g. converted from
    CHEMKIN input by pelelm_gb300.mech.chemkin) in name order."""
    import json
    names = []
    for f in sorted(os.listdir(DATA)):
        if not f.endswith(".json") or f.count(".") != 1:
            continue
        try:
            with open(os.path.join(DATA, f)) as fh:
                d = json.load(fh)
        except (OSError, ValueError):
            continue
        if isinstance(d, dict) and "species" in d and "reactions" in d:
            names.append(f[:-5])
    first = [n for n in ("lidryer_syn", "drm19_syn", "gri_syn") if n in names]
    return first + [n for n in names if n not in first]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pelelm_gb300")
    return p


def generate_sources() -> list:
    """Mechanism headers, tables, per-mechanism units and the registry list; returns the
    generated unit paths. The oracle's flat file is written for a mechanism that lacks one."""
    from .mech import codegen
    from .workloads import load_mechanism
    gen = os.path.join(CSRC, "gen")
    names = mechanism_names()
    codegen.main(gen, names=names)
    codegen.write_tables(gen, names=names)
    units = codegen.write_units(gen, names)
    for n in names:
        flat = os.path.join(DATA, f"{n}.mech")
        if not os.path.exists(flat):
            load_mechanism(n).to_flat(flat)
    # the exp64 constants are committed (their generator needs mpmath, absent on some hosts)
    if not os.path.exists(os.path.join(gen, "exp64_table.cuh")):
        subprocess.check_call([sys.executable, os.path.join(CSRC, "gen_exp64.py")])
    return units


def _sources_newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    units = [os.path.join(CSRC, u) for u in UNITS] + generate_sources()
    deps = [os.path.join(dp, f) for dp, _, fs in os.walk(CSRC) for f in fs
            if f.endswith((".cu", ".cuh", ".h", ".cpp", ".inc"))]
    deps.append(os.path.join(ROOT, "include", "pelelm_gb300.h"))
    if not force and not _sources_newer(LIB, deps):
        return LIB
    objs = []

    def compile_unit(src):
        u = os.path.basename(src)
        obj = os.path.join(BUILD, os.path.splitext(u)[0] + ".o")
        cmd = [nvcc(), *NVFLAGS, *ARCH, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        return obj, r.stderr

    # the largest units first, so the longest compile starts at once
    units.sort(key=lambda p: -os.path.getsize(p) if os.path.basename(p).startswith("unit_") else 0)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(units), os.cpu_count() or 1))) as ex:
        for obj, log in ex.map(compile_unit, units):
            objs.append(obj)
            if verbose and log:
                print(log)
    tmp = LIB + ".tmp"
    subprocess.check_call([nvcc(), *ARCH, "-shared", "-o", tmp, *objs])
    os.replace(tmp, LIB)
    return LIB


def build_oracle() -> str:
    subprocess.check_call(["make", "-s", "-C", os.path.join(ROOT, "oracle")])
    return os.path.join(ROOT, "oracle", "liboracle.so")


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
