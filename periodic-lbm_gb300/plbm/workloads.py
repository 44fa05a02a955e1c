"""Named workloads of the library, run from the command line (for timing
and for profilers such as ncu, which need one process per workload).

    PYTHONPATH=periodic-lbm_gb300 python -m plbm.workloads grid --n 2048 [--kind bgk]
        [--storage f64] [--math hybrid] [--streaming lbm] [--steps 3] [--warmup 3]
    ... batched --grids 64 [--storage f64] [--math hybrid] [--threads 128] [--persistent]
    ... plugin  --n 2048 [--storage f64] [--kind bgk]

Each builds its state (seeded TGV plus noise), runs `warmup` steps, then
`steps` timed steps on its own stream, and prints one JSON line with the
device time per step (CUDA events) and MLUPS.
"""
from __future__ import annotations

import argparse
import json
import math
import time


def _events(torch):
    return torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def run_grid(args) -> dict:
    import torch
    from . import LatticeGrid, cases
    n = args.n
    rho, ux, uy = cases.tgv_with_noise(n, u0=0.05, sigma=1e-4, seed=1234, nu=(0.6 - 0.5) / 3.0)
    st = torch.cuda.Stream()
    g = LatticeGrid(n, n, storage=args.storage, collision=args.kind, math=args.math, streaming=args.streaming)
    g.set_stream(st.cuda_stream)
    if args.streaming == "lbm":
        g.set_relaxation(1.0 / 0.6, 0.25)
    else:
        g.set_properties(0.05, 0.3)
    g.set_pdf_to_equilibrium(rho, ux, uy)
    g.perform_lbm_step(args.warmup)
    torch.cuda.synchronize()
    e0, e1 = _events(torch)
    e0.record(st)
    g.perform_lbm_step(args.steps)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    g.close()
    return {"workload": "grid", "n": n, "kind": args.kind, "storage": args.storage, "math": args.math,
            "streaming": args.streaming, "ms_per_step": ms, "mlups": n * n / (ms * 1e-3) / 1e6}


def run_batched(args) -> dict:
    import torch
    from . import batched
    b = batched.build_tgv_batch(args.grids, 2024, args.storage)
    b.set_math(args.math if args.storage == "f64" else "fma")
    s = b.schedule
    s.threads, s.persistent = args.threads, int(args.persistent)
    for i in range(len(s.ty)):
        s.ty[i] = min(s.ty[i], args.threads) if args.threads >= 32 else 32
    b.schedule = s
    st = torch.cuda.Stream()
    b.set_stream(st.cuda_stream)
    b.run(args.warmup)
    b.synchronize()
    e0, e1 = _events(torch)
    e0.record(st)
    b.run(args.steps)
    e1.record(st)
    b.synchronize()
    ms = e0.elapsed_time(e1) / max(args.steps, 1)
    cells = b.cells
    sched = b.schedule.as_dict()
    b.close()
    return {"workload": "batched", "grids": args.grids, "cells": cells, "storage": args.storage,
            "math": args.math, "schedule": sched, "ms_per_step": ms, "mlups": cells / (ms * 1e-3) / 1e6}


def run_plugin(args) -> dict:
    from .plugin import SimPlugin, make_params
    from .studies import TGVStudy
    n = args.n
    k = 2 * math.pi / n
    case = TGVStudy((n, n), umax=0.05, k=(k, k), nu=0.02)
    p0, u0 = case.solution(0.0)
    sim = SimPlugin()
    sim.init((n, n), 1.0, p0, u0, params=make_params(kind=args.kind, storage=args.storage, math=args.math))
    omega = 1.0 / (3 * 0.02 + 0.5)
    sim.steps(omega, args.warmup)
    sim.synchronize()
    # the plugin runs on its own stream: host clock around a synchronize
    t0 = time.perf_counter()
    sim.steps(omega, args.steps)
    sim.synchronize()
    ms = (time.perf_counter() - t0) * 1e3 / max(args.steps, 1)
    sim.free()
    return {"workload": "plugin", "n": n, "kind": args.kind, "storage": args.storage, "math": args.math,
            "ms_per_step": ms,
            "mlups": n * n / (ms * 1e-3) / 1e6}


def main(argv=None) -> None:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("workload", choices=["grid", "batched", "plugin"])
    ap.add_argument("--n", type=int, default=2048)
    ap.add_argument("--grids", type=int, default=64)
    ap.add_argument("--threads", type=int, default=128, help="batched: threads per CTA")
    ap.add_argument("--persistent", action="store_true", help="batched: one cooperative launch")
    ap.add_argument("--kind", default="bgk", choices=["bgk", "trt", "rr"])
    ap.add_argument("--storage", default="f64", choices=["f64", "f32dev", "f16dev"])
    ap.add_argument("--math", default="fma", choices=["fma", "strict", "hybrid", "df64"])
    ap.add_argument("--streaming", default="lbm")
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    args = ap.parse_args(argv)
    out = {"grid": run_grid, "batched": run_batched, "plugin": run_plugin}[args.workload](args)
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
