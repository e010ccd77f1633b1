#!/usr/bin/env python
"""Chemistry cells/sec per dt_react of the GB300 reactor on the AMR-like LiDryer workload.

Workload (one "step" = one advance of every cell of every box over dt_react):
  LiDryer-shaped H2/O2 mechanism (9 species, 21 reactions; synthetic, structure-matched),
  120 boxes with sides in {8,16,32,64} = 2,154,496 cells, dt_react = 1e-5 s, rtol 1e-6,
  atol 1e-10, N(0, 1e2^2) kg/m^3/s species forcing (realizable, zero net mass) and
  N(0, 1e8^2) W/m^3 energy forcing. Inputs are seeded synthetic states (no dataset exists).

Arms:
  default            the GB300 reactor through its C ABI (pgb_reactor_react_boxes), one
                     persistent work-stealing launch per step over all boxes.
  --impl reference   the CPU CVODE-class restatement of the reference reactor (the oracle) on
                     all host cores, timed on a bounded sample of the same workload.

Timing: W warm-up steps, then K timed steps, each bracketed by a barrier and
torch.cuda.synchronize() with CUDA events on the launch stream; the device state (577 MB)
exceeds L2 (129 MB) and is restored from a pristine copy between steps (untimed). `e2e`
repeats the steps from pinned host memory with the H2D input copies and D2H result copies
inside the timed region.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "chemistry cells/sec per dt_react"
UNIT = "cells/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb", choices=["gb", "reference"])
    p.add_argument("--config", default="lidryer_amr120")
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64-line", action="store_true")
    p.add_argument("--cpu-sample", type=int, default=0,
                   help="cells timed on the CPU (0 = the whole workload, ~10 s on 16 cores)")
    return p.parse_args()


# ---------------------------------------------------------------- distributed plumbing
def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if ws > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        backend = "nccl" if args.impl == "gb" else "gloo"
        dist.init_process_group(backend=backend, rank=rank, world_size=ws)
        pg = dist
    return ws, rank, local, pg


def barrier(pg, device=None):
    if pg is not None:
        if device is not None:
            pg.barrier(device_ids=[device])
        else:
            pg.barrier()


def allmax(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def allsum(pg, x):
    if pg is None:
        return x
    import torch
    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    pg.all_reduce(t)
    return float(t.item())


# ---------------------------------------------------------------- clocks
class ClockSampler:
    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def start(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- workload
def build_workload(cfg_name, seed):
    from pelelm_gb300.workloads import CONFIGS, box_layout, make_cells, to_box_arena
    cfg = CONFIGS[cfg_name]
    cs = make_cells(cfg, seed=seed)
    lay = box_layout(cfg.boxes)
    arenas = {
        "rY": to_box_arena(lay, cs.rY), "rY_src": to_box_arena(lay, cs.rYsrc),
        "T": to_box_arena(lay, cs.T[:, None]), "rEner": to_box_arena(lay, cs.rE[:, None]),
        "rEner_src": to_box_arena(lay, cs.rEsrc[:, None]),
    }
    return cfg, cs, lay, arenas


def box_views(torch, lay, dev, ns):
    """BoxArrays over device arenas (component-major block per box, one box after another)."""
    from pelelm_gb300.reactor import BoxArrays
    out = []
    for b, s in enumerate(lay.sides):
        c0, c1 = int(lay.cell_offset[b]), int(lay.cell_offset[b + 1])

        def v(name, nc):
            return dev[name][c0 * nc:c1 * nc].view(nc, s, s, s)

        out.append(BoxArrays(((0, 0, 0), (s - 1, s - 1, s - 1)), v("rY", ns), v("rY_src", ns), v("T", 1),
                             v("rEner", 1), v("rEner_src", 1), v("FC", 1), None))
    return out


def run_gb(args, ws, rank, local, pg):
    import torch
    from pelelm_gb300 import _lib
    from pelelm_gb300.mech.opcount import FLOPS_PER_TRANSCENDENTAL, rhs_flops, rhs_ops
    from pelelm_gb300.reactor import ReactorBase
    from pelelm_gb300.workloads import load_mechanism

    torch.cuda.set_device(local)
    dev_index = local
    cfg, cs, lay, arenas = build_workload(args.config, seed=rank)
    mech = load_mechanism(cfg.mech)
    ns, ncell = mech.ns, lay.ncell
    lib = _lib.lib()
    import ctypes as C
    peak = C.c_double()
    _lib.check(lib.pgb_fp64_peak_tflops(20000, C.byref(peak)), "fp64 peak")
    fp64_peak = peak.value

    stream = torch.cuda.Stream()
    fields = ["rY", "rY_src", "T", "rEner", "rEner_src"]
    pristine = {k: torch.from_numpy(arenas[k]).to("cuda") for k in fields}
    work = {k: v.clone() for k, v in pristine.items()}
    work["FC"] = torch.zeros(ncell, dtype=torch.float64, device="cuda")
    views = box_views(torch, lay, work, ns)

    def make_reactor(precision):
        r = ReactorBase.create("ReactorCvode", cfg.mech,
                               f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.precision={precision} gb.graph=1")
        r.init(2, 1)
        return r

    def restore():
        for k in fields:
            work[k].copy_(pristine[k])
        work["FC"].zero_()

    def timed_steps(r, nsteps, warm):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        for _ in range(warm):
            restore()
            with torch.cuda.stream(stream):
                r.react_boxes(views, cfg.dt, 0.0, stream=stream)
            torch.cuda.synchronize()
        total = 0.0
        sampler = ClockSampler(dev_index)
        sampler.start()
        for i in range(nsteps):
            restore()
            torch.cuda.synchronize()
            barrier(pg, dev_index)
            with torch.cuda.stream(stream):
                ev[i][0].record(stream)
                r.react_boxes(views, cfg.dt, 0.0, stream=stream)
                ev[i][1].record(stream)
            torch.cuda.synchronize()
            barrier(pg, dev_index)
            total += ev[i][0].elapsed_time(ev[i][1]) / 1e3
        clocks = sampler.stop()
        return total, clocks, r.stats()

    r = make_reactor(args.precision)
    t_kern, clocks, st = timed_steps(r, args.steps, args.warmup)
    t_max = allmax(pg, t_kern)
    cells_all = allsum(pg, float(ncell * args.steps))
    value = cells_all / t_max
    ms_per_step = 1e3 * t_max / args.steps
    nfe_per_step = st["nfe"]
    flops_rhs = rhs_flops(mech)
    ops, trans = rhs_ops(mech)
    achieved = flops_rhs * nfe_per_step / (t_kern / args.steps) / 1e12
    hist = st["hist"]

    # ---- e2e: pinned host inputs -> H2D -> advance -> D2H of the results, all timed
    host_in = {k: torch.from_numpy(arenas[k]).pin_memory() for k in fields}
    out_fields = ["rY", "T", "rEner", "FC"]
    host_out = {k: torch.empty_like(work[k], device="cpu").pin_memory() for k in out_fields}
    h2d = sum(v.numel() * 8 for v in host_in.values())
    d2h = sum(v.numel() * 8 for v in host_out.values())
    e2e_total = 0.0
    for i in range(args.warmup + args.steps):
        torch.cuda.synchronize()
        barrier(pg, dev_index)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            for k in fields:
                work[k].copy_(host_in[k], non_blocking=True)
            work["FC"].zero_()
            r.react_boxes(views, cfg.dt, 0.0, stream=stream)
            for k in out_fields:
                host_out[k].copy_(work[k], non_blocking=True)
            e1.record(stream)
        torch.cuda.synchronize()
        barrier(pg, dev_index)
        if i >= args.warmup:
            e2e_total += e0.elapsed_time(e1) / 1e3
    e2e_value = allsum(pg, float(ncell * args.steps)) / allmax(pg, e2e_total)
    nfail = int(st["nfail"])
    r.close()

    extra = {}
    if not args.no_fp64_line and args.precision != "fp64":
        r64 = make_reactor("fp64")
        t64, _, st64 = timed_steps(r64, max(1, min(args.steps, 2)), 1)
        extra["fp64_plain"] = {"cells_per_s": ncell * max(1, min(args.steps, 2)) / t64,
                               "ms_per_step": 1e3 * t64 / max(1, min(args.steps, 2)),
                               "nfe_per_step": st64["nfe"]}
        r64.close()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(cfg, cs, args.cpu_sample or ncell)

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32",
            "data": "synthetic (seeded states; synthetic structure-matched LiDryer-shaped mechanism)",
            "config": {"workload": "lidryer_amr120: LiDryer-shaped H2/O2 (9 sp, 21 rx), 120 boxes "
                                   "{8,16,32,64}^3 = 2,154,496 cells, dt_react 1e-5 s, rtol 1e-6, "
                                   "atol 1e-10, realizable N(0,1e2^2) kg/m^3/s + N(0,1e8^2) W/m^3 forcing",
                       "precision": args.precision, "cells_per_gpu": ncell,
                       "l2": "inputs (577 MB of state) larger than L2; state restored between steps",
                       "launch": "one persistent work-stealing kernel per step, CUDA-graph replay"},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp64_peak,
                         # DRAM bytes per launch: ncu capture of a 131,072-cell launch (22.8 MB,
                         # profiles/bdf_reactor_kernel_lidryer_131k.txt) scaled by cells
                         "traffic": 22.81e6 * ncell / 131072,
                         "what": f"rate evaluation: {flops_rhs} algorithmic FP64 flops per RHS "
                                 f"({ops} ops + {trans} transcendentals x {FLOPS_PER_TRANSCENDENTAL}) "
                                 f"x {nfe_per_step} RHS evaluations per step / kernel time",
                         "peak_source": "measured in this run: pgb_fp64_peak_tflops (DFMA, full grid)"},
            "stats": {"nst_per_cell": st["nst"] / ncell, "nfe_per_cell": st["nfe"] / ncell,
                      "nje_per_cell": st["nje"] / ncell, "max_steps_cell": st["max_nst"], "nfail": nfail,
                      "steps_hist_log2": hist},
            "clocks": clocks,
            "gpu_launches": args.steps,
            **extra,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------------- CPU (oracle) legs
def cpu_baseline(cfg, cs, sample, nthreads=0):
    """The oracle (C++ CVODE-class restatement, OpenMP) on a seeded uniform subsample."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from pelelm_gb300.workloads import mech_path
    O.build()
    om = O.OracleMech(mech_path(cfg.mech))
    n = cs.T.size
    rng = np.random.default_rng(99)
    idx = np.sort(rng.choice(n, size=min(sample, n), replace=False))
    cores = nthreads or O.max_threads()
    t0 = time.perf_counter()
    out = om.react(cs.rY[idx], cs.rYsrc[idx], cs.T[idx], cs.rE[idx], cs.rEsrc[idx], cs.mask[idx],
                   cfg.dt, cfg.rtol, cfg.atol, nthreads=cores)
    dt = time.perf_counter() - t0
    return {"value": idx.size / dt, "unit": UNIT, "cores": cores, "kind": "port",
            "sample": f"{idx.size} cells drawn uniformly (seed 99) from the same workload; "
                      f"{dt:.2f} s wall on {cores} threads", "nfail": int(out[4])}


def run_reference(args, ws, rank, pg):
    if rank != 0:
        return
    from pelelm_gb300.workloads import CONFIGS, make_cells
    cfg = CONFIGS[args.config]
    cs = make_cells(cfg, seed=0)
    # each step: a quarter of the workload (about 3 s on 16 cores), so K + W steps stay in minutes
    sample = args.cpu_sample or cfg.ncell // 4
    vals = []
    for i in range(args.warmup + args.steps):
        res = cpu_baseline(cfg, cs, sample)
        if i >= args.warmup:
            vals.append(res)
    value = float(np.mean([v["value"] for v in vals]))
    cores = vals[-1]["cores"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sample / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": "synthetic (seeded states; synthetic structure-matched LiDryer-shaped mechanism)",
            "config": {"workload": "lidryer_amr120 (bounded sample per step)", "cells_per_step": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{sample} cells per step, uniform subsample of the 2,154,496-cell "
                                       "workload; the reference's own CVODE reactor is not in the "
                                       "reference tree, so its C++ restatement (oracle/) runs"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    ws, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank, pg)
    else:
        run_gb(args, ws, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
