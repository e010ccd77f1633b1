"""Small reactor advance for profiling (ncu) and quick timing of one mechanism/config.

    python -m pelelm_gb300.profile_case --config lidryer_amr120 --cells 32768 [--precision mixed]

Builds `cells` seeded cells of the config (cubic boxes of 32^3, the last one partial is
padded into a smaller box), runs `--reps` advances through the C ABI and prints the CUDA-event
time of each. State is restored between advances.
"""
from __future__ import annotations

import argparse
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--config", default="lidryer_amr120")
    p.add_argument("--cells", type=int, default=32768)
    p.add_argument("--precision", default="mixed")
    p.add_argument("--reps", type=int, default=2)
    p.add_argument("--options", default="")
    args = p.parse_args()

    import numpy as np
    import torch

    from pelelm_gb300.reactor import BoxArrays, ReactorBase
    from pelelm_gb300.workloads import CONFIGS, box_layout, make_cells, to_box_arena

    cfg = CONFIGS[args.config]
    cs = make_cells(cfg, args.cells, seed=0)
    ns = cs.rY.shape[1]
    side = 32
    nfull = args.cells // side ** 3
    sides = [side] * nfull
    rest = args.cells - nfull * side ** 3
    shapes = [(side, side, side)] * nfull
    if rest:
        shapes.append((rest, 1, 1))
    lay_off = np.cumsum([0] + [a * b * c for a, b, c in shapes])
    fields = {"rY": (cs.rY, ns), "rY_src": (cs.rYsrc, ns), "T": (cs.T[:, None], 1),
              "rEner": (cs.rE[:, None], 1), "rEner_src": (cs.rEsrc[:, None], 1)}
    pristine = {}
    for k, (a, nc) in fields.items():
        blocks = [a[lay_off[b]:lay_off[b + 1]].T.reshape(-1) for b in range(len(shapes))]
        pristine[k] = torch.tensor(np.concatenate(blocks), device="cuda")
    work = {k: v.clone() for k, v in pristine.items()}
    work["FC"] = torch.zeros(args.cells, dtype=torch.float64, device="cuda")
    boxes = []
    for b, (nx, ny, nz) in enumerate(shapes):
        c0, c1 = int(lay_off[b]), int(lay_off[b + 1])

        def v(name, nc):
            return work[name][c0 * nc:c1 * nc].view(nc, nz, ny, nx)

        boxes.append(BoxArrays(((0, 0, 0), (nx - 1, ny - 1, nz - 1)), v("rY", ns), v("rY_src", ns),
                               v("T", 1), v("rEner", 1), v("rEner_src", 1), v("FC", 1), None))
    r = ReactorBase.create("ReactorCvode", cfg.mech,
                           f"ode.rtol={cfg.rtol} ode.atol={cfg.atol} gb.precision={args.precision} "
                           + args.options)
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
    print(json.dumps({"config": args.config, "cells": args.cells, "precision": args.precision,
                      "ms": times, "cells_per_s": args.cells / (min(times) / 1e3),
                      "nfe_per_cell": st["nfe"] / args.cells, "nst_per_cell": st["nst"] / args.cells,
                      "nje_per_cell": st["nje"] / args.cells,
                      "nfail": st["nfail"], "nretry": st["nretry"]}))


if __name__ == "__main__":
    main()
