"""Benchmark of the D2Q9 periodic stream-collide hot path on GB300.

Headline workload: plain single-grid bandwidth bench, D2Q9 BGK, tau = 0.6,
8192 x 8192 periodic grid, binary64 SoA f(ld,nx,0:8), two lattices (9.66 GB,
75x the 129 MB L2, so no L2 flush is needed between steps).  Initial state:
Taylor-Green vortex u0 = 0.05 (k = 2 pi / 8192) plus seeded i.i.d.
N(0, 1e-4^2) velocity noise, f at equilibrium.  A step is one
perform_lbm_step (one fused pull-stream + collide kernel) over the grid.
The headline arithmetic is PLBM_MATH_HYBRID (binary64 storage, one binary64
FMA per population on an exact integer bracket, exact integer moments); the
straight binary64 kernel is measured beside it ("variants.fp64_native").

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--n 8192] [--kind bgk|trt|rr] [--storage f64|f32dev|f16dev]
                    [--math fma|strict|hybrid] [--no-variants] [--no-cpu-baseline]
                    [--suite mixed|fields|adjoint]

Prints one JSON line (rank 0).  --impl reference times the reference's
algorithm on the host cores instead: the C restatement of the Fortran
(two passes per step, stream then collide, OpenMP over all host threads).
--suite mixed runs the mixed-precision study (shear layer, 8192^2, tau 0.52,
velocity L2 error of binary32/binary16 deviation storage against binary64 at
steps 1000/5000/20000) and prints its own JSON line; --suite fields times the
two field kernels around the job (equilibrium, moments) on device-resident
fields, integer forms and reference expressions ("variants.field_kernels");
--suite adjoint times the config-5 adjoint alone (1024^2, T = 2000, K = 45,
binary32 storage; "variants.adjoint_f32dev"; --adj-n / --adj-steps shrink it).
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
PKG = ROOT / "periodic-lbm_gb300"
for _p in (str(ROOT), str(PKG)):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

# Algorithmic HBM bytes per cell update of the fused step (read 9 + write 9
# populations) by storage.
BYTES_PER_CELL = {"f64": 144, "f32dev": 72, "f16dev": 36}
# DRAM bytes per cell update measured by ncu (dram__bytes_read.sum +
# dram__bytes_write.sum of one launch / cells) on a 2048^2 capture of the same
# kernel, scaled by the cell count: profiles/k_step_*_2048_fullset.md.
NCU_TRAFFIC_PER_CELL = {("f64", "bgk", "hybrid"): 132.6, ("f64", "trt", "hybrid"): 132.4,
                        ("f64", "rr", "hybrid"): 133.0, ("f64", "bgk", "fma"): 132.4}
FALLBACK_HBM_GBS = 6800.0


def measured_peak_gbs() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        v = float(json.loads(p.read_text())["hbm_gbs"])
        return v, "measured"
    except Exception:
        return FALLBACK_HBM_GBS, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    FIELDS = ("uuid,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, uuid: str | None):
        self.uuid = (uuid or "").lower()
        self.lines: list[str] = []
        self.proc = None
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
            return
        self.t = threading.Thread(target=self._read, daemon=True)
        self.t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            if self.uuid and not (parts[0].lower().endswith(self.uuid[-12:]) or self.uuid in parts[0].lower()):
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def initial_fields(n: int):
    from plbm import cases
    return cases.tgv_with_noise(n, u0=0.05, sigma=1e-4, seed=1234, nu=(0.6 - 0.5) / 3.0)


def cpu_reference_run(n: int, kind: str, omega: float, steps: int, warmup: int, fields=None) -> dict:
    """Time the C restatement of the reference (two passes per step, OpenMP)."""
    from oracle import oracle as O
    kinds = {"bgk": O.BGK, "trt": O.TRT, "rr": O.RR}
    rho, ux, uy = fields if fields is not None else initial_fields(n)
    f2 = np.empty((2, 9, n, O.pad16(n)))
    f2[0] = 0.0
    f2[1] = O.set_pdf_to_equilibrium(rho, ux, uy)
    del rho, ux, uy
    iold, inew = 2, 1
    if warmup:
        iold, inew = O.perform_lbm_step(f2, n, iold, inew, kinds[kind], omega, 0.25, warmup, fast=True)
    t0 = time.perf_counter()
    iold, inew = O.perform_lbm_step(f2, n, iold, inew, kinds[kind], omega, 0.25, steps, fast=True)
    dt = time.perf_counter() - t0
    return {"seconds": dt, "steps": steps, "mlups": n * n * steps / dt / 1e6,
            "threads": O.num_threads(fast=True)}


def cpu_model() -> str:
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True).stdout
        for line in out.splitlines():
            if line.startswith("Model name"):
                return line.split(":", 1)[1].strip()
    except Exception:
        pass
    return "unknown"


def workload_config(args) -> dict:
    esize = {"f64": 8, "f32dev": 4, "f16dev": 2}[args.storage]
    return {"workload": f"plain single-grid bandwidth bench: D2Q9 {args.kind.upper()} tau={args.tau} "
                        f"{args.n}x{args.n} periodic, {args.storage} SoA two-lattice, TGV u0=0.05 + N(0,1e-4^2) noise",
            "grid": [args.n, args.n], "collision": args.kind, "tau": args.tau, "storage": args.storage,
            "math": args.math, "layout": "f(ld,nx,0:8) y-fastest, ld=pad16(ny)",
            "l2_policy": f"inputs larger than L2 (two lattices of {2 * 9 * args.n * args.n * esize / 1e9:.2f} GB "
                         "vs 129 MB L2); no flush",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    os.environ.setdefault("OMP_PROC_BIND", "close")
    n = args.n
    omega = 1.0 / args.tau
    r = cpu_reference_run(n, args.kind, omega, args.steps, args.warmup)
    sample = (f"{n}x{n} D2Q9 {args.kind.upper()} binary64, {args.steps} timed steps after {args.warmup} "
              f"warm-up, two passes per step (lbm_stream then collide_{args.kind}), "
              f"{r['threads']} OpenMP threads on {cpu_model()}")
    line = {
        "metric": "MLUPS", "value": r["mlups"], "unit": "MLUPS", "impl": "reference",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * r["seconds"] / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded TGV + noise)",
        "config": workload_config(args),
        "cpu_baseline": {"value": r["mlups"], "unit": "MLUPS", "cores": r["threads"], "kind": "port",
                         "sample": sample},
        "e2e": {"value": r["mlups"], "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
def time_grid_steps(torch, n, storage, kind, math_mode, omega, steps, warmup, fields):
    """Device-resident MLUPS of one grid configuration (CUDA events, own stream)."""
    from plbm import LatticeGrid
    stream = torch.cuda.Stream()
    g = LatticeGrid(n, n, storage=storage, collision=kind, math=math_mode)
    g.set_stream(stream.cuda_stream)
    g.set_relaxation(omega, 0.25)
    g.set_pdf_to_equilibrium(*fields)
    g.perform_lbm_step(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.perform_lbm_step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    g.close()
    return ms / steps


def field_kernels_variant(torch, n, fields, peak, reps=5):
    """Device time of the two field kernels around the job on device-resident
    (ny,nx) fields: plbm_equilibrium_device (24 B in, 72 B out per cell) and
    plbm_macros_device (72 B in, 24 B out), per arithmetic: the integer forms
    of hybrid grids and the reference's binary64 expressions (FMA grids).
    CUDA events on the grid's stream, median of reps; inputs exceed L2."""
    from plbm import LatticeGrid, _lib
    lib = _lib.load()
    stream = torch.cuda.Stream()
    dev = [torch.from_numpy(np.ascontiguousarray(a)).to("cuda") for a in fields]
    out = [torch.empty_like(dev[0]) for _ in range(3)]
    bytes_per_cell = 96.0
    res = {"workload": f"{n}^2 cells, rho/ux/uy (ny,nx) binary64 on the device <-> one binary64 lattice",
           "algorithmic_bytes_per_cell": bytes_per_cell}
    for mm in ("hybrid", "fma"):
        g = LatticeGrid(n, n, collision="bgk", math=mm)
        g.set_stream(stream.cuda_stream)
        times = {}
        for name in ("equilibrium", "macros"):
            def launch():
                if name == "equilibrium":
                    _lib.check(lib.plbm_equilibrium_device(g.handle, g.iold, *(d.data_ptr() for d in dev)))
                else:
                    _lib.check(lib.plbm_macros_device(g.handle, g.iold, *(o.data_ptr() for o in out)))
            launch()
            torch.cuda.synchronize()
            ts = []
            for _ in range(reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                launch()
                e1.record(stream)
                torch.cuda.synchronize()
                ts.append(e0.elapsed_time(e1))
            ms = float(np.median(ts))
            gbs = bytes_per_cell * n * n / (ms * 1e-3) / 1e9
            times[name] = {"ms": ms, "achieved_gbs": gbs, "frac_of_measured_hbm": gbs / peak}
        if mm == "hybrid":
            # moments of the equilibrium against the rho it was built from
            m = [o.double().cpu().numpy() for o in out]
            times["rho_roundtrip_max_abs"] = float(np.max(np.abs(m[0] - fields[0])))
        g.close()
        res["integer_forms" if mm == "hybrid" else "reference_expressions"] = times
    del dev, out
    torch.cuda.empty_cache()
    return res


def time_scheme_steps(torch, n, scheme, math_mode, steps, warmup, fields):
    """Device MLUPS of perform_lbm_step with a finite-volume / finite-difference
    streaming scheme (dt = 0.3, nu = 0.05) and BGK."""
    from plbm import LatticeGrid
    stream = torch.cuda.Stream()
    g = LatticeGrid(n, n, collision="bgk", math=math_mode, streaming=scheme)
    g.set_stream(stream.cuda_stream)
    g.set_properties(0.05, 0.3)
    g.set_pdf_to_equilibrium(*fields)
    g.perform_lbm_step(warmup)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.perform_lbm_step(steps)
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    g.close()
    return ms / steps


def time_plugin_steps(n, math_mode, steps, warmup, kind="bgk"):
    """Milliseconds per step of the sim/ plugin ABI (c_plbmgpu_*) at n^2,
    binary64 storage, host clock around c_plbmgpu_steps + c_plbmgpu_synchronize."""
    from plbm.plugin import SimPlugin, make_params
    from plbm.studies import TGVStudy
    k = 2 * math.pi / n
    p0, u0 = TGVStudy((n, n), umax=0.05, k=(k, k), nu=0.02).solution(0.0)
    sim = SimPlugin()
    sim.init((n, n), 1.0, p0, u0, params=make_params(kind=kind, math=math_mode))
    del p0, u0
    omega = 1.0 / (3 * 0.02 + 0.5)
    sim.steps(omega, warmup)
    sim.synchronize()
    t0 = time.perf_counter()
    sim.steps(omega, steps)
    sim.synchronize()
    dt = time.perf_counter() - t0
    sim.free()
    return dt * 1e3 / steps


# ---- replicas: one process per GPU, independent grids (no data-path collective)
def max_over_ranks(x: float, world: int, device: str = "cuda") -> float:
    """The slowest rank's time (the job ends when the last replica ends)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_mlups(cells_per_rank: int, steps: int, world: int, seconds_max: float) -> float:
    """Whole-job throughput: the cell updates of all replicas over the slowest rank's time."""
    return world * cells_per_rank * steps / seconds_max / 1e6


def variant_entry(n, storage, ms_step, peak):
    mlups = n * n / (ms_step * 1e-3) / 1e6
    gbs = mlups * 1e6 * BYTES_PER_CELL[storage] / 1e9
    return {"value": mlups, "unit": "MLUPS", "ms_per_step": ms_step, "achieved_gbs": gbs, "frac_hbm": gbs / peak,
            "bytes_per_cell": BYTES_PER_CELL[storage]}


MIXED_CONFS = (("f32dev", "hybrid"), ("f32dev", "fma"), ("f16dev", "hybrid"), ("f16dev", "fma"))


def mixed_precision_errors(torch, n, tau, checkpoints):
    """Velocity L2 error of binary32/binary16 deviation storage (compensated
    "hybrid" and plain binary32 collision) against the binary64 run, shear
    layer k=80, delta=0.05, u0=0.04, BGK tau."""
    from plbm import LatticeGrid, cases
    rho, ux, uy = cases.shear_layer(n, n, float(n), 0.04, 80.0, 0.05)
    grids = {}
    for st, mm in (("f64", "hybrid"),) + MIXED_CONFS:
        g = LatticeGrid(n, n, storage=st, collision="bgk", math=mm)
        g.set_relaxation(1.0 / tau, 0.25)
        g.set_pdf_to_equilibrium(rho, ux, uy)
        grids[(st, mm)] = g
    out = {f"{st}/{mm}": {} for st, mm in MIXED_CONFS}
    done = 0
    for c in checkpoints:
        for g in grids.values():
            g.perform_lbm_step(c - done)
        done = c
        _, u64, v64 = grids[("f64", "hybrid")].update_macros()
        den = float(np.sum(u64 * u64 + v64 * v64))
        for st, mm in MIXED_CONFS:
            _, u, v = grids[(st, mm)].update_macros()
            out[f"{st}/{mm}"][str(c)] = math.sqrt(float(np.sum((u - u64) ** 2 + (v - v64) ** 2)) / den)
    for g in grids.values():
        g.close()
    return out


def batched_variant(torch, storage, steps, math="fma", both=True):
    """Config 4: 512 uneven grids advanced `steps` steps per CUDA-graph launch,
    with the schedule the autotuner picked; with both=True the other mode
    (one persistent cooperative launch vs one launch per step) is timed with
    the same threads too, so the tuner's choice is on record."""
    from plbm import autotune, batched
    b = batched.build_tgv_batch(512, 2024, storage)
    b.set_math(math)
    _, rep = autotune.tune(b, steps=10, reps=1, use_cache=True, final_steps=100)
    stream = torch.cuda.Stream()
    b.set_stream(stream.cuda_stream)
    cells = b.cells

    def timed(sched):
        b.schedule = batched.Schedule.from_dict(sched)
        b.capture(steps)
        b.launch_graph()
        b.synchronize()
        if b.steps % 2:
            b.capture(steps)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.launch_graph()
        e1.record(stream)
        b.synchronize()
        return e0.elapsed_time(e1)

    tuned = dict(rep["schedule"])
    ms = timed(tuned)
    mlups = cells * steps / (ms * 1e-3) / 1e6
    modes = {("persistent" if tuned["persistent"] else "per_step"): mlups}
    if both:
        other = dict(tuned, persistent=1 - int(tuned["persistent"]), ctas_per_sm=0)
        ms_o = timed(other)
        modes["persistent" if other["persistent"] else "per_step"] = cells * steps / (ms_o * 1e-3) / 1e6
    b.close()
    return {"value": mlups, "unit": "MLUPS", "grids": 512, "cells": cells, "math": math, "steps_per_graph": steps,
            "ms_per_step": ms / steps, "schedule": tuned, "persistent": int(tuned["persistent"]),
            "schedule_cached": rep.get("cached", False), "mlups_by_mode": modes,
            "tuner": "fastest of threads x {persistent, per-step} x ty x CTAs/SM on 10-step trials, then the "
                     "winner against the other mode's best on 100 steps",
            "achieved_gbs": mlups * 1e6 * BYTES_PER_CELL[storage] / 1e9}


def adjoint_variant(torch, storage, n=1024, T=2000, K=45):
    from plbm import cases
    from plbm.autograd import Adjoint
    ux, uy = cases.divergence_free_modes(n, 16, 8, 0.01, seed=1)
    tx, ty = cases.divergence_free_modes(n, 16, 8, 0.01, seed=2)
    u0 = torch.tensor(np.stack([ux, uy]), device="cuda")
    tgt = torch.tensor(np.stack([tx, ty]), device="cuda")

    def timed(math_mode):
        a = Adjoint(n, n, T, K, storage, math=math_mode)
        uT = a.forward(u0, 1 / 0.8)
        a.backward(uT - tgt)
        torch.cuda.synchronize()
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        uT = a.forward(u0, 1 / 0.8)
        e[1].record()
        a.backward(uT - tgt)
        e[2].record()
        torch.cuda.synchronize()
        f_ms, b_ms = e[0].elapsed_time(e[1]), e[1].elapsed_time(e[2])
        mem = a.memory_bytes()
        g, dom = a.backward(uT - tgt)
        a.close()
        return f_ms, b_ms, mem, g, dom

    f_ms, b_ms, mem, g32, dom32 = timed("fma")
    fc_ms, bc_ms, _, gc, domc = timed("hybrid")
    # the binary64 model's adjoint gradient of the same problem: the binary32
    # storage gradients' errors against it (dL/du0 norm-wise, dL/dtau)
    a64 = Adjoint(n, n, T, K, "f64")
    uT64 = a64.forward(u0, 1 / 0.8)
    g64, dom64 = a64.backward(uT64 - tgt)
    a64.close()
    torch.cuda.synchronize()

    def errs(g, dom):  # dL/dtau = -dL/domega tau^2: the same relative error
        return {"du0_l2": float(torch.linalg.norm(g - g64) / torch.linalg.norm(g64)),
                "dtau": abs(dom - dom64) / abs(dom64)}

    return {"grid": [n, n], "steps": T, "checkpoint_every": K, "storage": storage, "forward_ms": f_ms,
            "backward_ms": b_ms, "adjoint_over_forward": b_ms / f_ms, "device_GB": mem / 1e9,
            "grad_rel_err_f32_vs_f64": dict(errs(g32, dom32), against="binary64 discrete adjoint of the same problem"),
            "compensated_reverse_step": {"forward_ms": fc_ms, "backward_ms": bc_ms, "adjoint_over_forward": bc_ms / fc_ms,
                                         "grad_rel_err_f32_vs_f64": errs(gc, domc),
                                         "math": "plbm_adjoint_set_math(PLBM_MATH_HYBRID)"}}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=8192)
    ap.add_argument("--kind", default="bgk", choices=["bgk", "trt", "rr"])
    ap.add_argument("--tau", type=float, default=0.6)
    ap.add_argument("--storage", default="f64", choices=["f64", "f32dev", "f16dev"])
    ap.add_argument("--math", default=None, choices=["fma", "strict", "hybrid"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU-baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--suite", default=None, choices=["mixed", "fields", "adjoint"])
    ap.add_argument("--adj-n", type=int, default=1024, help="--suite adjoint: grid edge")
    ap.add_argument("--adj-steps", type=int, default=2000, help="--suite adjoint: time steps T")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.math is None:
        args.math = "hybrid" if args.storage == "f64" else "fma"

    if args.impl == "reference":
        run_reference(args)
        return

    import torch
    import torch.distributed as dist

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")

    from plbm import LatticeGrid, _lib
    try:
        _lib.load()
    except RuntimeError:
        import __graft_entry__ as ge
        ge.build()
        _lib.load()

    if args.suite == "mixed":
        if rank == 0:
            errs = mixed_precision_errors(torch, args.n, 0.52, (1000, 5000, 20000))
            print(json.dumps({"suite": "mixed", "workload": f"shear layer {args.n}^2 BGK tau=0.52 k=80 delta=0.05 "
                              "u0=0.04", "velocity_l2_vs_f64": errs}), flush=True)
        return

    if args.suite == "adjoint":
        if rank == 0:
            print(json.dumps({"suite": "adjoint", **adjoint_variant(torch, "f32dev", n=args.adj_n, T=args.adj_steps)}),
                  flush=True)
        return

    if args.suite == "fields":
        if rank == 0:
            peak = measured_peak_gbs()[0]
            print(json.dumps({"suite": "fields", **field_kernels_variant(torch, args.n, initial_fields(args.n),
                                                                          peak)}), flush=True)
        return

    n, omega = args.n, 1.0 / args.tau
    fields = initial_fields(n)
    # a dedicated stream: the kernels and the timing events share it
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    g = LatticeGrid(n, n, storage=args.storage, collision=args.kind, math=args.math)
    g.set_stream(stream.cuda_stream)
    g.set_relaxation(omega, 0.25)
    g.set_pdf_to_equilibrium(*fields)

    def barrier():
        if world > 1:
            dist.barrier()

    # ---- device-resident timing: K fused steps --------------------------------
    g.perform_lbm_step(args.warmup)
    torch.cuda.synchronize()
    props = torch.cuda.get_device_properties(local)
    sampler = ClockSampler(str(getattr(props, "uuid", "")))
    sampler.start()
    time.sleep(0.3)
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    g.perform_lbm_step(args.steps)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms = e0.elapsed_time(e1)
    clocks = sampler.stop()
    ms_max = max_over_ranks(ms, world)
    cells = n * n
    mlups = job_mlups(cells, args.steps, world, ms_max * 1e-3)

    # ---- end to end through the C ABI with host buffers -------------------------
    # One job as the reference's drivers run it (app/main_taylor_green.f90:
    # 100-147): pinned host rho/ux/uy -> plbm_set_pdf_to_equilibrium, K
    # plbm_perform_lbm_step(grid,1) calls, plbm_update_macros to pinned host
    # rho/ux/uy.  Copies are inside the timed region.
    lib = _lib.load()
    h = g.handle
    pinned = lambda: torch.empty((n, n), dtype=torch.float64, pin_memory=True).numpy()  # noqa: E731
    host_in = [pinned() for _ in range(3)]
    for dst, src in zip(host_in, fields):
        dst[...] = src
    host_m = [pinned() for _ in range(3)]

    def e2e_job(start):
        """One untimed run of the job (first use of the pinned buffers), then
        the median of three timed runs."""
        times = []
        for rep in range(4):
            barrier()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            start()
            for _ in range(args.steps):
                _lib.check(lib.plbm_perform_lbm_step(h, 1))
            _lib.check(lib.plbm_update_macros(h, *[m.ctypes.data for m in host_m]))
            torch.cuda.synchronize()
            dt = time.perf_counter() - t0
            barrier()
            if rep:
                times.append(max_over_ranks(dt, world))
        return job_mlups(n * n, args.steps, world, sorted(times)[1])

    e2e_mlups = e2e_job(lambda: _lib.check(lib.plbm_set_pdf_to_equilibrium(h, *[m.ctypes.data for m in host_in])))
    h2d = 3 * n * n * 8
    d2h = 3 * n * n * 8
    # The same job started from a full lattice instead (pinned host
    # f(ld,nx,0:8) -> plbm_upload): 9 ld/ny times the input bytes.
    ld = g.ld
    host_f = torch.empty((9, n, ld), dtype=torch.float64, pin_memory=True).numpy()
    host_f[...] = g.download(g.iold)
    e2e_f_mlups = e2e_job(lambda: _lib.check(lib.plbm_upload(h, host_f.ctypes.data, g.iold)))
    h2d_f = 9 * n * ld * 8
    g.close()
    del host_f, host_m, host_in

    if rank != 0:
        if world > 1:
            dist.destroy_process_group()
        return

    peak, peak_kind = measured_peak_gbs()
    per_launch_s = ms_max * 1e-3 / args.steps
    algo_bytes = BYTES_PER_CELL[args.storage] * cells
    achieved = algo_bytes / per_launch_s / 1e9
    traffic = NCU_TRAFFIC_PER_CELL.get((args.storage, args.kind, args.math))
    line = {
        "metric": "MLUPS", "value": mlups, "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": {"f64": "f64", "f32dev": "f32", "f16dev": "f16"}[args.storage],
        "data": "synthetic (seeded TGV + noise, no dataset)",
        "config": workload_config(args),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic * cells if traffic else None,
                     "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_cell": BYTES_PER_CELL[args.storage]},
        "e2e": {"value": e2e_mlups, "unit": "MLUPS", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps,
                "job": "plbm_set_pdf_to_equilibrium(pinned rho, ux, uy) + K x plbm_perform_lbm_step(1) + "
                       "plbm_update_macros(pinned)",
                "timing": "host clock around the whole job; one untimed run, median of three",
                "from_lattice_upload": {"value": e2e_f_mlups, "h2d_bytes_per_step": h2d_f / args.steps,
                                        "job": "plbm_upload(pinned f) + K x plbm_perform_lbm_step(1) + "
                                               "plbm_update_macros(pinned)"}},
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if not args.no_variants:
        torch.cuda.empty_cache()
        var = {}
        var["fp64_native"] = variant_entry(n, "f64", time_grid_steps(torch, n, "f64", args.kind, "fma", omega, 20, 3,
                                                                    fields), peak)
        for other in ("bgk", "trt", "rr"):
            if other == args.kind:
                continue
            for mm in ("hybrid", "fma"):
                e = variant_entry(n, "f64", time_grid_steps(torch, n, "f64", other, mm, omega, 20, 3, fields), peak)
                e["workload"] = f"{n}^2 {other.upper()} binary64, {mm} arithmetic, same state and tau"
                var[f"fp64_{other}_{mm}"] = e
        for scheme in ("fdm_bardow", "fdm_sofonea"):
            for mm in ("hybrid", "strict"):
                e = variant_entry(n, "f64", time_scheme_steps(torch, n, scheme, mm, 10, 2, fields), peak)
                e["workload"] = (f"{n}^2 BGK with grid%streaming => stream_{scheme}, dt=0.3 nu=0.05, "
                                 + ("fused stencil + hybrid collision" if mm == "hybrid" else
                                    "reference expressions, two passes"))
                var[f"scheme_{scheme}_{mm}"] = e
        for mm in ("hybrid", "fma"):
            e = variant_entry(n, "f64", time_plugin_steps(n, mm, 20, 3), peak)
            e["workload"] = f"{n}^2 sim/ plugin ABI (c_plbmgpu_*), binary64 BGK, {mm} arithmetic, host clock"
            var[f"plugin_f64_{mm}"] = e
        var["fp32dev"] = variant_entry(n, "f32dev", time_grid_steps(torch, n, "f32dev", args.kind, "fma", omega, 50, 3,
                                                                   fields), peak)
        if args.kind == "bgk":
            var["fp32dev_compensated"] = variant_entry(
                n, "f32dev", time_grid_steps(torch, n, "f32dev", "bgk", "hybrid", omega, 50, 3, fields), peak)
        var["fp16dev"] = variant_entry(n, "f16dev", time_grid_steps(torch, n, "f16dev", args.kind, "fma", omega, 50, 3,
                                                                   fields), peak)
        mp = mixed_precision_errors(torch, n, 0.52, (1000, 5000, 20000))
        var["mixed_precision_l2_vs_f64"] = {
            "workload": f"shear layer {n}^2 BGK tau=0.52 k=80 delta=0.05 u0=0.04, velocity L2 error against "
                        "the binary64 (hybrid) run at steps 1000/5000/20000", **mp,
            "meets_1e-6": {k: max(v.values()) <= 1e-6 for k, v in mp.items()}}
        var["fp32dev"]["velocity_l2_vs_f64"] = mp["f32dev/fma"]
        var["fp32dev"]["meets_1e-6"] = max(mp["f32dev/fma"].values()) <= 1e-6
        if "fp32dev_compensated" in var:
            var["fp32dev_compensated"]["velocity_l2_vs_f64"] = mp["f32dev/hybrid"]
            var["fp32dev_compensated"]["meets_1e-6"] = max(mp["f32dev/hybrid"].values()) <= 1e-6
        var["fp16dev"]["velocity_l2_vs_f64"] = mp["f16dev/fma"]
        var["fp16dev"]["meets_1e-6"] = max(mp["f16dev/fma"].values()) <= 1e-6
        var["field_kernels"] = field_kernels_variant(torch, n, fields, peak)
        var["batched_f64"] = batched_variant(torch, "f64", 1000, "hybrid")
        var["batched_f64_fma"] = batched_variant(torch, "f64", 50, both=False)
        var["batched_f32dev"] = batched_variant(torch, "f32dev", 1000)
        var["adjoint_f32dev"] = adjoint_variant(torch, "f32dev")
        line["variants"] = var
    if not args.no_cpu_baseline:
        # bounded sample of the same workload: estimate one step, then size the run
        one = cpu_reference_run(n, args.kind, omega, 1, 1, fields)
        steps = max(1, min(50, int(args.cpu_seconds / max(one["seconds"], 1e-3))))
        r = cpu_reference_run(n, args.kind, omega, steps, 0, fields)
        line["cpu_baseline"] = {
            "value": r["mlups"], "unit": "MLUPS", "cores": r["threads"], "kind": "port",
            "sample": f"{n}x{n} {args.kind.upper()} binary64, {steps} steps (two passes each) of the C "
                      f"restatement, {r['threads']} OpenMP threads on {cpu_model()}"}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
