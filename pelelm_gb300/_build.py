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
UNITS = ["reactor.cu", "peak.cu", "noalloc.cu", "partition.cpp", "mlp.cu", "surrogate_io.cu", "mech_lidryer_syn.cu", "mech_drm19_syn.cu",
         "mech_gri_syn.cu"]


def nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build pelelm_gb300")
    return p


def generate_sources() -> None:
    from .mech import codegen
    gen = os.path.join(CSRC, "gen")
    codegen.main(gen, names=("lidryer_syn", "drm19_syn", "gri_syn"))
    codegen.write_tables(gen, names=("lidryer_syn", "drm19_syn", "gri_syn"))
    # the exp64 constants are committed (their generator needs mpmath, absent on some hosts)
    if not os.path.exists(os.path.join(gen, "exp64_table.cuh")):
        subprocess.check_call([sys.executable, os.path.join(CSRC, "gen_exp64.py")])


def _sources_newer(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    generate_sources()
    deps = [os.path.join(dp, f) for dp, _, fs in os.walk(CSRC) for f in fs
            if f.endswith((".cu", ".cuh", ".h", ".cpp"))]
    deps.append(os.path.join(ROOT, "include", "pelelm_gb300.h"))
    if not force and not _sources_newer(LIB, deps):
        return LIB
    objs = []

    def compile_unit(u):
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, os.path.splitext(u)[0] + ".o")
        cmd = [nvcc(), *NVFLAGS, *ARCH, "-c", src, "-o", obj]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {u}:\n{r.stderr}")
        return obj, r.stderr

    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(UNITS), os.cpu_count() or 1))) as ex:
        for obj, log in ex.map(compile_unit, UNITS):
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
