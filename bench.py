#!/usr/bin/env python
"""Chemistry cells/sec per dt_react: learned surrogate + BDF fallback vs the plain GPU BDF.

Default workload (one "step" = one advance of every cell of every box over dt_react):
  drm19-shaped CH4/air mechanism (21 species, 84 reactions; synthetic, structure-matched),
  96 x 32^3 + 256 x 16^3 = 2^22 cells (the surrogate benchmark's inference size), T = 300 + 1900 c,
  phi ~ U[0.6, 1.4], dt_react = 1e-5 s, rtol 1e-6, atol 1e-10, N(0, 1e2^2) kg/m^3/s species
  forcing (realizable, zero net mass) and N(0, 1e8^2) W/m^3 energy forcing. Inputs are seeded
  synthetic states (no dataset exists). The reactor runs the trained surrogate
  (pelelm_gb300/data/drm19_syn.pgbs) over every cell; cells failing its checks, plus a 1% audit
  sample, are advanced by the GPU BDF in the same CUDA graph. Reported beside it: the same
  workload through the plain GPU BDF (mixed precision, and FP64 throughout), the share of the
  step in each kernel, the error of the result against the FP64 oracle at rtol 1e-10
  (stratified subsample), and compact lines (plain GPU BDF mixed and FP64 with their rooflines,
  CPU oracle beside them) for the LiDryer 32^3 box, the LiDryer 120-box AMR workload and a
  65,536-cell subset of the GRI-shaped workload. `--config lidryer_amr120 --surrogate none`
  gives the plain BDF on the 2,154,496-cell LiDryer-shaped AMR workload as the headline.

Arms:
  default            the GB300 reactor through its C ABI (pgb_reactor_react_boxes).
  --impl reference   the CPU CVODE-class restatement of the reference reactor (the oracle) on
                     all host cores, timed on a bounded sample of the same workload.

Timing: W warm-up steps, then K timed steps, each bracketed by a barrier and
torch.cuda.synchronize() with CUDA events on the launch stream; the device state (2.3 GB for
drm19_4M) exceeds L2 (129 MB) and is restored from a pristine copy between steps (untimed).
`e2e` repeats min(K, 3) steps from pinned host memory with the H2D input copies and D2H result
copies inside the timed region.
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

METRIC = "chemistry cells/sec per dt_react: surrogate+fallback vs GPU BDF at \u22641 K error"
UNIT = "cells/s"


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=2)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb", choices=["gb", "reference"])
    p.add_argument("--config", default="drm19_4M")
    p.add_argument("--surrogate", default="pelelm_gb300/data/drm19_syn.pgbs",
                   help="trained surrogate file, or 'none' for the plain GPU BDF")
    p.add_argument("--no-error-check", action="store_true")
    p.add_argument("--error-sample", type=int, default=4096)
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-fp64-line", action="store_true")
    p.add_argument("--no-pareto", action="store_true",
                   help="skip the surrogate's looser operating points (acceptance vs tolerance)")
    p.add_argument("--no-extras", action="store_true",
                   help="skip the compact lines of the other benchmark configurations")
    p.add_argument("--cpu-sample", type=int, default=0,
                   help="cells timed on the CPU (0 = the whole workload, ~10 s on 16 cores)")
    p.add_argument("--profile-case", action="store_true",
                   help="small advance for ncu captures: --cells seeded cells of --config in 32^3 "
                        "boxes, --reps advances, one JSON line with their CUDA-event times")
    p.add_argument("--cells", type=int, default=32768)
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--options", default="", help="extra reactor options (profile case)")
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
class Shard:
    """This rank's boxes of the global box list and their host arenas (component-major block per
    box, boxes one after another).

    The global list holds one copy of the configuration's boxes per rank (per-GPU work fixed as
    ranks are added: weak scaling); global box g is a cube of side cfg.boxes[g % nbox] whose cells
    are drawn from their own stream seeded (0, g), so any rank can build any box. Boxes go to
    ranks by pelelm_gb300.sharding.partition_boxes over `weights` (cell counts before the first
    advance, the boxes' FC sums after it)."""

    def __init__(self, cfg, ws, rank, weights=None):
        from pelelm_gb300.sharding import partition_boxes
        from pelelm_gb300.workloads import box_layout, make_box_cells, to_box_arena
        self.sides_global = list(cfg.boxes) * ws
        w = (np.array([s ** 3 for s in self.sides_global], dtype=np.float64) if weights is None
             else np.asarray(weights, dtype=np.float64))
        self.ranks, self.load = partition_boxes(w, ws)
        self.boxes = [g for g in range(len(self.sides_global)) if self.ranks[g] == rank]
        self.cs = make_box_cells(cfg, self.sides_global, self.boxes, seed=0)
        self.lay = box_layout([self.sides_global[g] for g in self.boxes])
        cs = self.cs
        self.arenas = {
            "rY": to_box_arena(self.lay, cs.rY), "rY_src": to_box_arena(self.lay, cs.rYsrc),
            "T": to_box_arena(self.lay, cs.T[:, None]), "rEner": to_box_arena(self.lay, cs.rE[:, None]),
            "rEner_src": to_box_arena(self.lay, cs.rEsrc[:, None]),
        }

    @property
    def ncell(self):
        return self.lay.ncell

    def fc_weights(self, fc):
        """{global box: sum of its cells' FC} from the flat device FC array of this shard."""
        from pelelm_gb300.sharding import fc_weights
        off = self.lay.cell_offset
        w = fc_weights([fc[int(off[i]):int(off[i + 1])] for i in range(len(self.boxes))])
        return {g: float(x) for g, x in zip(self.boxes, w)}


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

    from pelelm_gb300.workloads import CONFIGS
    torch.cuda.set_device(local)
    dev_index = local
    cfg = CONFIGS[args.config]
    shard = Shard(cfg, ws, rank)
    mech = load_mechanism(cfg.mech)
    ns = mech.ns
    surrogate = args.surrogate if args.surrogate != "none" else None
    if surrogate and not os.path.isabs(surrogate):
        surrogate = os.path.join(ROOT, surrogate)
    lib = _lib.lib()
    import ctypes as C
    peak = C.c_double()
    _lib.check(lib.pgb_fp64_peak_tflops(20000, C.byref(peak)), "fp64 peak")
    fp64_peak = peak.value
    peaks = measured_peaks()

    stream = torch.cuda.Stream()
    fields = ["rY", "rY_src", "T", "rEner", "rEner_src"]
    pristine, work, views = {}, {}, []

    def upload():
        pristine.clear()
        work.clear()
        pristine.update({k: torch.from_numpy(shard.arenas[k]).to("cuda") for k in fields})
        work.update({k: v.clone() for k, v in pristine.items()})
        work["FC"] = torch.zeros(shard.ncell, dtype=torch.float64, device="cuda")
        views[:] = box_views(torch, shard.lay, work, ns)

    upload()
    base_opts = f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.graph=1 gb.autotune=1"

    def make_reactor(precision, extra=""):
        r = ReactorBase.create("ReactorCvode", cfg.mech, f"{base_opts} gb.precision={precision} {extra}")
        r.init(2, 1)
        return r

    def restore():
        for k in fields:
            work[k].copy_(pristine[k])
        work["FC"].zero_()

    def timed_steps(r, nsteps, warm, clocks=True):
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(nsteps)]
        for _ in range(warm):
            restore()
            with torch.cuda.stream(stream):
                r.react_boxes(views, cfg.dt, 0.0, stream=stream)
            torch.cuda.synchronize()
        total = 0.0
        sampler = ClockSampler(dev_index)
        if clocks:
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
        return total, (sampler.stop() if clocks else None), r.stats()

    sg_opts = f"gb.surrogate={surrogate}" if surrogate else ""
    r = make_reactor(args.precision, sg_opts)
    rebalance = None
    if ws > 1:
        # the first warm-up advance runs the cell-count partition; every rank then shares its
        # boxes' FC sums (host objects, between advances) and all ranks re-partition the global
        # box list by that cost, as PeleLM's getFuncCountDM does with the previous FuncCount
        restore()
        with torch.cuda.stream(stream):
            r.react_boxes(views, cfg.dt, 0.0, stream=stream)
        torch.cuda.synchronize()
        mine = shard.fc_weights(work["FC"])
        allw = [None] * ws
        pg.all_gather_object(allw, mine)
        weights = np.zeros(len(shard.sides_global))
        for d in allw:
            for g, x in d.items():
                weights[int(g)] = x
        load_cells = shard.load
        shard = Shard(cfg, ws, rank, weights)
        upload()
        rebalance = {"by": "FC sums of the first warm-up advance", "boxes_global": len(shard.sides_global),
                     "max_over_mean_load": float(shard.load.max() / max(shard.load.mean(), 1e-300)),
                     "cell_partition_max_over_mean_cells": float(load_cells.max() / max(load_cells.mean(), 1e-300))}
    t_step, clocks, st = timed_steps(r, args.steps, max(args.warmup - (1 if ws > 1 else 0), 1))
    ncell, cs, lay, arenas = shard.ncell, shard.cs, shard.lay, shard.arenas
    sst = r.surrogate_stats() if surrogate else None
    tuning = r.tuning()
    family = tuned_family(tuning, cfg.mech)
    t_max = allmax(pg, t_step)
    value = allsum(pg, float(ncell * args.steps)) / t_max
    ms_per_step = 1e3 * t_max / args.steps
    out_state = {k: work[k].clone() for k in ("rY", "T", "FC")} if surrogate else None

    # ---- e2e: pinned host inputs -> H2D -> advance -> D2H of the results, all timed (the
    # reactor is warm from the steps above: one untimed e2e pass, then K timed)
    host_in = {k: torch.from_numpy(arenas[k]).pin_memory() for k in fields}
    out_fields = ["rY", "T", "rEner", "FC"]
    host_out = {k: torch.empty_like(work[k], device="cpu").pin_memory() for k in out_fields}
    h2d = sum(v.numel() * 8 for v in host_in.values())
    d2h = sum(v.numel() * 8 for v in host_out.values())
    e2e_total = 0.0
    n_e2e = max(1, min(args.steps, 3))  # cells/s is size- and step-independent at this scale
    for i in range(1 + n_e2e):
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
        if i >= 1:
            e2e_total += e0.elapsed_time(e1) / 1e3
    e2e_value = allsum(pg, float(ncell * n_e2e)) / allmax(pg, e2e_total)
    r.close()

    flops_rhs = rhs_flops(mech)
    ops, trans = rhs_ops(mech)
    extra = {}
    if surrogate:
        # the same workload through the plain GPU BDF (same precision), and the surrogate kernel
        # alone (every gate open: no cell reaches the BDF) to split the step between kernels
        rp = make_reactor(args.precision)
        n_plain = max(1, min(args.steps, 2))
        t_plain, _, st_plain = timed_steps(rp, n_plain, 1, clocks=False)
        rp.close()
        ra = make_reactor(args.precision, sg_opts + " gb.sg.audit=0 gb.sg.mis=1e30 gb.sg.cons=1e30 "
                          "gb.sg.disT=1e30 gb.sg.disY=1e30 gb.sg.neg=1e30 gb.sg.ood_margin=1e30")
        t_sg, _, _ = timed_steps(ra, 3, 2, clocks=False)
        t_sg /= 3
        ra.close()
        plain_cps = allsum(pg, float(ncell * n_plain)) / allmax(pg, t_plain)
        t_bdf = max(t_step / args.steps - t_sg, 1e-9)
        nfe = st["nfe"]
        achieved = flops_rhs * nfe / t_bdf / 1e12
        from pelelm_gb300.surrogate import read_pgbs
        d = read_pgbs(surrogate)
        mlp_flops = 2.0 * d["nmodel"] * sum(int(d["dims"][l]) * int(d["dims"][l + 1]) for l in range(d["nlayer"]))
        extra["plain_gpu_bdf"] = {"cells_per_s": plain_cps, "ms_per_step": 1e3 * t_plain / n_plain,
                                  "nfe_per_cell": st_plain["nfe"] / ncell, "precision": args.precision}
        extra["speedup_vs_plain_gpu_bdf"] = value / plain_cps
        extra["surrogate"] = {
            "file": os.path.relpath(surrogate, ROOT), "members": d["nmodel"],
            "accepted_frac": sst["accept"] / max(sst["ncell"], 1),
            "fallback_frac": sst["fallback"] / max(sst["ncell"], 1),
            "audit_frac": sst["audit"] / max(sst["ncell"], 1), "audit_bad": sst["audit_bad"],
            "audit_max_dT_K": sst["audit_max_dT"], "audit_max_dY": sst["audit_max_dY"],
            "rejected_by": {k: sst[k] for k in ("ood", "mis", "cons", "ens", "neg")},
            "bdf_work_saved_frac": 1.0 - nfe / max(st_plain["nfe"], 1),
            "kernel_ms": {"surrogate_inference": 1e3 * t_sg, "bdf_fallback_and_audit": 1e3 * t_bdf},
            "inference_roofline": {"bound": "tensor", "unit": "TFLOP/s",
                                   "achieved": mlp_flops * ncell / t_sg / 1e12,
                                   "peak": peaks.get("bf16_tflops"),
                                   "frac": (mlp_flops * ncell / t_sg / 1e12 / peaks["bf16_tflops"])
                                   if peaks.get("bf16_tflops") else None,
                                   "what": f"{mlp_flops:.0f} padded MMA flops per cell (ensemble of "
                                           f"{d['nmodel']}) / surrogate kernel time incl. featurise+gates",
                                   "peak_source": "MEASURED_PEAKS.json bf16 (cuBLAS burst) of measured"},
        }
        if rank == 0 and not args.no_error_check:
            extra["error_vs_fp64_oracle"] = error_vs_oracle(cfg, cs, lay, out_state, args.error_sample)
        if not args.no_pareto:
            extra["surrogate_pareto"] = surrogate_pareto(
                surrogate, make_reactor, sg_opts, timed_steps, work, plain_cps, ncell, pg, rank, cfg, cs, lay,
                args.error_sample, None if args.no_error_check else error_vs_oracle)
        dominant = f"{KERNEL_OF_FAMILY[family]} (fallback cells)"
    else:
        nfe = st["nfe"]
        achieved = flops_rhs * nfe / (t_step / args.steps) / 1e12
        dominant = KERNEL_OF_FAMILY[family]
    if not args.no_fp64_line and args.precision != "fp64":
        # the plain GPU BDF in FP64 throughout (the reference's own precision) on the same
        # workload: the like-for-like figure beside the mixed-precision one
        n64 = 1
        r64 = make_reactor("fp64")
        t64, _, st64 = timed_steps(r64, n64, 1, clocks=False)
        r64.close()
        extra["fp64_plain_gpu_bdf"] = {
            "cells_per_s": allsum(pg, float(ncell * n64)) / allmax(pg, t64), "ms_per_step": 1e3 * t64 / n64,
            "steps": n64, "warmup": 1, "nfe_per_cell": st64["nfe"] / ncell, "nfail": int(st64["nfail"]),
            "roofline_frac": flops_rhs * st64["nfe"] / (t64 / n64) / 1e12 / fp64_peak}

    if rank == 0 and cfg.mech != "gri_syn":
        extra["rate_evaluation"] = rates_roofline(torch, cfg, cs, stream, flops_rhs, fp64_peak)
    if rank == 0 and not args.no_extras:
        others = EXTRA_CONFIGS + ([] if args.config.startswith("drm19") else [("drm19_2M", None)])
        extra["other_configs"] = {name: config_extra(torch, name, ncells, stream, fp64_peak, cpu=not args.no_cpu_baseline)
                                  for name, ncells in others if name != args.config}

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        cpu = cpu_baseline(cfg, cs, args.cpu_sample or default_cpu_sample(cfg))

    if rank == 0:
        hist = st["hist"]
        line = {
            "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_per_step, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64" if args.precision == "fp64" else "f64+f32",
            "data": f"synthetic (seeded states; synthetic structure-matched {mech.name} mechanism)",
            "config": {"workload": WORKLOAD_TEXT.get(args.config, args.config) +
                       (" | learned surrogate (4x256 GELU BF16 MLP ensemble, fused inference) with "
                        "BDF fallback and 1% audit" if surrogate else " | plain GPU BDF"),
                       "precision": args.precision, "cells_per_gpu": ncell,
                       "sharding": ("one global box list (one copy of the configuration's boxes per "
                                    "rank), partitioned by pgb_partition_boxes: cell counts for the first "
                                    "warm-up advance, then the boxes' FC sums" if ws > 1 else
                                    "single rank: every box"),
                       **({"rebalance": rebalance} if rebalance else {}),
                       "l2": f"inputs ({ncell * (3 * ns + 5) * 8 / 1e6:.0f} MB of state) larger than L2; "
                             "state restored between steps",
                       "launch": "surrogate kernel -> persistent work-stealing BDF on the device fallback "
                                 "list -> audit kernel, one CUDA graph per step" if surrogate else
                                 "one persistent work-stealing kernel per step, CUDA-graph replay",
                       "autotune": tuning},
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                    "steps": n_e2e, "warmup": 1},
            "roofline": {"bound": "fp64", "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s",
                         "frac": achieved / fp64_peak,
                         # DRAM bytes per launch from an ncu capture of a smaller launch of the same
                         # kernel, scaled by cells (profiles/)
                         "traffic": (TRAFFIC_PER_CELL[(cfg.mech, family)] * (sst["fallback"] if surrogate else ncell)
                                     if (cfg.mech, family) in TRAFFIC_PER_CELL else None),
                         "kernel": dominant,
                         "what": f"rate evaluation: {flops_rhs} algorithmic FP64 flops per RHS "
                                 f"({ops} ops + {trans} transcendentals x {FLOPS_PER_TRANSCENDENTAL}) "
                                 f"x {nfe} RHS evaluations per step / BDF kernel time",
                         "peak_source": "measured in this run: pgb_fp64_peak_tflops (DFMA, full grid)"},
            "stats": {"nst_per_cell": st["nst"] / ncell, "nfe_per_cell": st["nfe"] / ncell,
                      "nje_per_cell": st["nje"] / ncell, "max_steps_cell": st["max_nst"], "nfail": int(st["nfail"]), "nretry": int(st["nretry"]),
                      "steps_hist_log2": hist},
            "clocks": clocks,
            # per step: [surrogate] + BDF (+ FP64 retry pass in mixed precision) + [audit]
            "gpu_launches": args.steps * ((2 if surrogate else 0) + (2 if args.precision == "mixed" else 1)),
            **extra,
        }
        if cpu:
            line["cpu_baseline"] = cpu
        print(json.dumps(line), flush=True)


def surrogate_pareto(surrogate, make_reactor, sg_opts, timed_steps, work, plain_cps, ncell, pg, rank, cfg, cs,
                     lay, sample, error_fn):
    """The surrogate at each calibrated operating point of its sidecar file (<file>.levels.json:
    1 K / 1e-4, 2 K / 3e-4, 5 K / 1e-3, 10 K / 3e-3): one warm-up and one timed advance of the
    whole workload each, the accepted fraction, the speed-up over the plain GPU BDF and the error
    of the accepted cells against the FP64 oracle at rtol 1e-10 (stratified subsample)."""
    with open(surrogate + ".levels.json") as f:
        levels = json.load(f)["levels"]
    out = []
    for lv in levels:
        opts = sg_opts + " " + " ".join(f"gb.sg.{k}={lv[k]!r}" for k in ("mis", "cons", "disT", "disY", "neg",
                                                                           "tol_T", "tol_Y"))
        r = make_reactor("mixed", opts)
        t, _, _ = timed_steps(r, 1, 1, clocks=False)
        sst = r.surrogate_stats()
        r.close()
        cps = allsum(pg, float(ncell)) / allmax(pg, t)
        pt = {"tol_T_K": lv["tol_T"], "tol_Y": lv["tol_Y"], "accepted_frac": sst["accept"] / max(sst["ncell"], 1),
              "cells_per_s": cps, "speedup_vs_plain_gpu_bdf": cps / plain_cps,
              "calibration_accepted_frac": lv.get("val_accept")}
        if error_fn is not None and rank == 0 and sst["accept"] > 0:
            e = error_fn(cfg, cs, lay, {k: work[k].clone() for k in ("rY", "T", "FC")}, sample)["surrogate_cells"]
            pt["accepted_cells_vs_oracle"] = e
            pt["within_tolerance"] = bool(e["max_dT_K"] <= lv["tol_T"] and e["max_dY"] <= lv["tol_Y"])
        out.append(pt)
    return out


# Compact lines for the other benchmark configurations: (config, cells; None = all). The
# GRI-shaped line runs a stated 65,536-cell subset of gri_1M (its BDF takes ~40 s per 2^20 cells).
# The drm19 2^21-cell plain configuration is the headline's plain_gpu_bdf leg (same state
# distribution on 2^22 cells), so it gets its own line only when the headline runs elsewhere.
# (configuration, cells): None = the whole configuration; an int = a subset in 16^3 boxes; a
# dict = a subset per precision (GRI: the FP64 pass is 8x slower; the mixed pass on a larger
# subset amortises the serial tail of the few cells that run to the step limit)
EXTRA_CONFIGS = [("lidryer_32cube", None), ("lidryer_amr120", None),
                 ("gri_1M", {"mixed": 262144, "fp64": 65536})]


def config_extra(torch, name, ncells, stream, fp64_peak, cpu=True, steps=1, warm=1):
    """Plain GPU BDF on one benchmark configuration (mixed and FP64, CUDA events on the launch
    stream, state restored between steps), its FP64 rate-evaluation roofline and, on a bounded
    sample, the CPU oracle beside it."""
    from pelelm_gb300.mech.opcount import rhs_flops
    from pelelm_gb300.reactor import BoxArrays, ReactorBase
    from pelelm_gb300.workloads import CONFIGS, box_layout, load_mechanism, make_cells, to_box_arena
    cfg = CONFIGS[name]
    mech = load_mechanism(cfg.mech)
    ns = mech.ns
    flops = rhs_flops(mech)
    out = {"workload": WORKLOAD_TEXT.get(name, name) +
           (" | subsets in 16^3 boxes (cells per precision below)" if ncells is not None else "")}
    cs = None
    for precision in ("mixed", "fp64"):
        nsub = ncells.get(precision) if isinstance(ncells, dict) else ncells
        if nsub is None:
            sides = list(cfg.boxes)
            cs = make_cells(cfg, seed=0)
        else:
            sides = [16] * (nsub // 4096)
            cs = make_cells(cfg, 4096 * len(sides), seed=0)
        lay = box_layout(sides)
        n = lay.ncell
        host = {"rY": cs.rY, "rY_src": cs.rYsrc, "T": cs.T[:, None], "rEner": cs.rE[:, None],
                "rEner_src": cs.rEsrc[:, None]}
        pristine = {k: torch.from_numpy(to_box_arena(lay, a)).to("cuda") for k, a in host.items()}
        work = {k: v.clone() for k, v in pristine.items()}
        work["FC"] = torch.zeros(n, dtype=torch.float64, device="cuda")
        views = box_views(torch, lay, work, ns)
        r = ReactorBase.create("ReactorCvode", cfg.mech, f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.graph=1 "
                               f"gb.precision={precision}")
        r.init(2, 1)
        t = 0.0
        for i in range(warm + steps):
            for k in pristine:
                work[k].copy_(pristine[k])
            work["FC"].zero_()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            with torch.cuda.stream(stream):
                e0.record(stream)
                r.react_boxes(views, cfg.dt, 0.0, stream=stream)
                e1.record(stream)
            torch.cuda.synchronize()
            if i >= warm:
                t += e0.elapsed_time(e1) / 1e3
        st = r.stats()
        r.close()
        out[precision] = {"cells": n, "subset": nsub is not None,
                          "cells_per_s": n * steps / t, "ms_per_step": 1e3 * t / steps, "steps": steps,
                          "warmup": warm, "nfe_per_cell": st["nfe"] / n, "nst_per_cell": st["nst"] / n,
                          "nfail": int(st["nfail"]), "nretry": int(st["nretry"]),
                          "roofline": {"bound": "fp64", "unit": "TFLOP/s",
                                       "achieved": flops * st["nfe"] / (t / steps) / 1e12, "peak": fp64_peak,
                                       "frac": flops * st["nfe"] / (t / steps) / 1e12 / fp64_peak,
                                       "what": f"{flops} FP64 flops per RHS x RHS evaluations / BDF time"}}
        del pristine, work, views
    if cpu:
        res = cpu_baseline(cfg, cs, min(cs.T.size, default_cpu_sample(cfg) // 4), single_core=False)
        out["cpu_oracle"] = {k: res[k] for k in ("value", "unit", "cores", "kind", "sample")}
    return out


def rates_roofline(torch, cfg, cs, stream, flops_rhs, fp64_peak, reps=5):
    """Instantaneous production rates (reactionRateRhoY: T from (rho h, Y), then omega-dot) of
    every cell of the workload in one launch of `rates_kernel`, MKS in/out, CUDA-event timed."""
    import numpy as np
    from pelelm_gb300.reactor import reaction_rates
    n, ns = cs.T.size, cs.rY.shape[1]
    rY = torch.tensor(np.ascontiguousarray(cs.rY.T) * 1e3, device="cuda").view(ns, 1, 1, n)
    rH = torch.tensor(cs.rE * 0.1, device="cuda").view(1, 1, 1, n)
    T = torch.tensor(cs.T, device="cuda").view(1, 1, 1, n)
    out = torch.empty_like(rY)
    box = ((0, 0, 0), (n - 1, 0, 0))
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(stream):
        for _ in range(3):
            reaction_rates(cfg.mech, box, rY, rH, T, None, out, stream=stream)
        e0.record(stream)
        for _ in range(reps):
            reaction_rates(cfg.mech, box, rY, rH, T, None, out, stream=stream)
        e1.record(stream)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1e3 / reps
    achieved = flops_rhs * n / t / 1e12
    return {"kernel": "rates_kernel", "cells": n, "ms_per_launch": 1e3 * t, "cells_per_s": n / t,
            "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
            "what": f"{flops_rhs} counted FP64 flops per cell (one RHS); the T-from-(rho h, Y) Newton "
                    "iterations before the rates are executed but not counted",
            "bytes_per_cell": 8 * (2 * ns + 2), "inputs_vs_l2": "inputs larger than L2"}


WORKLOAD_TEXT = {
    "lidryer_amr120": "lidryer_amr120: LiDryer-shaped H2/O2 (9 sp, 21 rx), 120 boxes {8,16,32,64}^3 = "
                      "2,154,496 cells, dt_react 1e-5 s, rtol 1e-6, atol 1e-10, realizable N(0,1e2^2) "
                      "kg/m^3/s + N(0,1e8^2) W/m^3 forcing",
    "drm19_2M": "drm19_2M: drm19-shaped CH4/air (21 sp, 84 rx), 48x32^3 + 128x16^3 = 2^21 cells, "
                "T = 300 + 1900 c, phi ~ U[0.6,1.4], dt_react 1e-5 s, rtol 1e-6, atol 1e-10, forcing as "
                "lidryer_amr120",
    "drm19_4M": "drm19_4M: drm19-shaped CH4/air (21 sp, 84 rx), the drm19_2M state distribution on "
                "96x32^3 + 256x16^3 = 2^22 cells, dt_react 1e-5 s, rtol 1e-6, atol 1e-10",
    "gri_1M": "gri_1M: GRI-shaped CH4/air (53 sp, 325 rx), 2x64^3 + 14x32^3 + 14x16^3 + 16x8^3 = 2^20 cells, "
              "T = 300 + 2100 c, phi ~ U[0.5,1.5], p ~ U[1,10] atm, dt_react 1e-5 s, rtol 1e-6, atol 1e-10, "
              "forcing as lidryer_amr120",
}

# DRAM bytes per cell of one BDF launch, per mechanism and kernel family (dram__bytes_read.sum +
# dram__bytes_write.sum of an ncu capture of a smaller launch of the same kernel, divided by its
# cells; profiles/)
TRAFFIC_PER_CELL = {("lidryer_syn", "thread"): 22.81e6 / 131072,
                    ("drm19_syn", "group"): (12.428544e6 + 0.0) / 32768,
                    ("drm19_syn", "warp"): (12.076800e6 + 0.017408e6) / 32768}
KERNEL_OF_FAMILY = {"thread": "bdf_reactor_kernel", "warp": "bdf_warp_kernel", "group": "bdf_group_kernel"}


def tuned_family(tuning: str, mech: str) -> str:
    """Kernel family the autotuner picked ("... -> group/8"), else the library's default for the
    mechanism's size (per thread up to 12 species, lane groups up to 31)."""
    if "->" in tuning:
        fam = tuning.rsplit("->", 1)[1].strip().split("/")[0]
        if fam in KERNEL_OF_FAMILY:
            return fam
    from pelelm_gb300.workloads import load_mechanism
    ns = load_mechanism(mech).ns
    return "thread" if ns <= 12 else "group" if ns + 1 <= 32 else "warp"


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return {}
    out = {}
    for k, v in d.items():
        if isinstance(v, (int, float)):
            out[k] = float(v)
    return out


def error_vs_oracle(cfg, cs, lay, out_state, sample):
    """Error of the step's result against the FP64 oracle at rtol 1e-10 on a subsample stratified
    by what the surrogate did (accepted cells and BDF cells, each spread uniformly over T)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    from pelelm_gb300.workloads import from_box_arena, mech_path
    O.build()
    ns = cs.rY.shape[1]
    rY = from_box_arena(lay, out_state["rY"].cpu().numpy(), ns)
    T = from_box_arena(lay, out_state["T"].cpu().numpy(), 1)
    FC = from_box_arena(lay, out_state["FC"].cpu().numpy(), 1)
    acc = np.nonzero(FC == 0.0)[0]
    fb = np.nonzero(FC != 0.0)[0]
    idx = []
    for grp in (acc, fb):
        if grp.size:
            order = grp[np.argsort(cs.T[grp], kind="stable")]
            k = min(order.size, sample // 2 if acc.size and fb.size else sample)
            idx.append(order[np.linspace(0, order.size - 1, k).astype(int)])
    idx = np.unique(np.concatenate(idx))
    om = O.OracleMech(mech_path(cfg.mech))
    t0 = time.perf_counter()
    tight = om.react(cs.rY[idx], cs.rYsrc[idx], cs.T[idx], cs.rE[idx], cs.rEsrc[idx], cs.mask[idx], cfg.dt,
                     1e-10, 1e-14, max_steps=200000)
    dt = time.perf_counter() - t0
    Yg = rY[idx] / rY[idx].sum(1, keepdims=True)
    Yo = tight[0] / tight[0].sum(1, keepdims=True)
    eT = np.abs(T[idx] - tight[1])
    eY = np.abs(Yg - Yo).max(1)
    a = np.isin(idx, acc)

    def summ(m):
        if not m.any():
            return None
        return {"n": int(m.sum()), "max_dT_K": float(eT[m].max()), "p99_dT_K": float(np.percentile(eT[m], 99)),
                "max_dY": float(eY[m].max()), "p99_dY": float(np.percentile(eY[m], 99))}

    return {"oracle": "oracle/ C++ BDF, FP64, rtol 1e-10, atol 1e-14", "oracle_s": round(dt, 2),
            "all": summ(np.ones_like(a)), "surrogate_cells": summ(a), "bdf_cells": summ(~a),
            "within_1K_1e-4": bool(eT.max() <= 1.0 and eY.max() <= 1e-4)}


def default_cpu_sample(cfg):
    # about 10-30 s of CPU work on the box's 16 cores
    return {"lidryer_syn": cfg.ncell, "drm19_syn": 131072, "gri_syn": 16384}.get(cfg.mech, 65536)


# ---------------------------------------------------------------- CPU (oracle) legs
def cpu_baseline(cfg, cs, sample, nthreads=0, single_core=True):
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
    res = {"value": idx.size / dt, "unit": UNIT, "cores": cores, "kind": "port",
           "sample": f"{idx.size} cells drawn uniformly (seed 99) from the same workload; "
                     f"{dt:.2f} s wall on {cores} threads", "nfail": int(out[4])}
    if single_core and cores > 1:
        # one core on a smaller sample (about 2 s), for the per-core rate
        n1 = max(256, min(idx.size, int(2.0 * idx.size / dt / cores)))
        i1 = idx[:n1]
        t0 = time.perf_counter()
        om.react(cs.rY[i1], cs.rYsrc[i1], cs.T[i1], cs.rE[i1], cs.rEsrc[i1], cs.mask[i1], cfg.dt, cfg.rtol,
                 cfg.atol, nthreads=1)
        res["single_core"] = {"value": n1 / (time.perf_counter() - t0), "cells": int(n1)}
    return res


def run_reference(args, ws, rank, pg):
    if rank != 0:
        return
    from pelelm_gb300.workloads import CONFIGS
    cfg = CONFIGS[args.config]
    cs = Shard(cfg, 1, 0).cs  # the GB300 arm's single-rank workload
    # each step: a bounded sample (a few seconds on 16 cores), so K + W steps stay in minutes
    sample = args.cpu_sample or default_cpu_sample(cfg) // 4
    vals = []
    for i in range(args.warmup + args.steps):
        res = cpu_baseline(cfg, cs, sample, single_core=False)
        if i >= args.warmup:
            vals.append(res)
    value = float(np.mean([v["value"] for v in vals]))
    cores = vals[-1]["cores"]
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": 1e3 * sample / value, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "impl": "reference",
            "data": f"synthetic (seeded states; synthetic structure-matched {cfg.mech} mechanism)",
            "config": {"workload": WORKLOAD_TEXT.get(args.config, args.config) + " | CPU CVODE-class BDF "
                                   "(bounded sample per step)", "cells_per_step": sample},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"{sample} cells per step, uniform subsample of the {cfg.ncell}-cell "
                                       "workload; the reference's own CVODE reactor is not in the "
                                       "reference tree, so its C++ restatement (oracle/) runs"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_profile_case(args):
    """A small reactor advance of one config, for ncu captures and quick timings: `cells` seeded
    cells in 32^3 boxes (a remainder in one (rest, 1, 1) box), `reps` advances through the C ABI
    from a restored state, each timed with CUDA events; prints one JSON line."""
    import torch
    from pelelm_gb300.reactor import BoxArrays, ReactorBase
    from pelelm_gb300.workloads import CONFIGS, make_cells

    cfg = CONFIGS[args.config]
    n = args.cells
    cs = make_cells(cfg, n, seed=0)
    ns = cs.rY.shape[1]
    side = 32
    nfull = n // side ** 3
    shapes = [(side, side, side)] * nfull
    if n - nfull * side ** 3:
        shapes.append((n - nfull * side ** 3, 1, 1))
    off = np.cumsum([0] + [a * b * c for a, b, c in shapes])
    fields = {"rY": (cs.rY, ns), "rY_src": (cs.rYsrc, ns), "T": (cs.T[:, None], 1),
              "rEner": (cs.rE[:, None], 1), "rEner_src": (cs.rEsrc[:, None], 1)}
    pristine = {k: torch.tensor(np.concatenate([a[off[b]:off[b + 1]].T.reshape(-1) for b in range(len(shapes))]),
                                device="cuda") for k, (a, nc) in fields.items()}
    work = {k: v.clone() for k, v in pristine.items()}
    work["FC"] = torch.zeros(n, dtype=torch.float64, device="cuda")
    boxes = []
    for b, (nx, ny, nz) in enumerate(shapes):
        c0, c1 = int(off[b]), int(off[b + 1])

        def v(name, nc):
            return work[name][c0 * nc:c1 * nc].view(nc, nz, ny, nx)

        boxes.append(BoxArrays(((0, 0, 0), (nx - 1, ny - 1, nz - 1)), v("rY", ns), v("rY_src", ns),
                               v("T", 1), v("rEner", 1), v("rEner_src", 1), v("FC", 1), None))
    r = ReactorBase.create("ReactorCvode", cfg.mech, f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} "
                           f"gb.precision={args.precision} {args.options}")
    r.init(2, 1)
    stream = torch.cuda.Stream()
    times = []
    for _ in range(args.reps):
        for k in pristine:
            work[k].copy_(pristine[k])
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        with torch.cuda.stream(stream):
            e0.record(stream)
            r.react_boxes(boxes, cfg.dt, 0.0, stream=stream)
            e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    st = r.stats()
    r.close()
    print(json.dumps({"config": args.config, "cells": n, "precision": args.precision, "options": args.options,
                      "ms": times, "cells_per_s": n / (min(times) / 1e3), "nfe_per_cell": st["nfe"] / n,
                      "nst_per_cell": st["nst"] / n, "nje_per_cell": st["nje"] / n, "nfail": st["nfail"],
                      "nretry": st["nretry"]}), flush=True)


def main():
    args = parse()
    if args.profile_case:
        run_profile_case(args)
        return
    ws, rank, local, pg = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, ws, rank, pg)
    else:
        run_gb(args, ws, rank, local, pg)
    if pg is not None:
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
