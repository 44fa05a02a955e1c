"""Benchmark of the D2Q9 periodic stream-collide hot path on GB300.

Workload (default): plain single-grid bandwidth bench, D2Q9 BGK, tau = 0.6,
8192 x 8192 periodic grid, binary64 SoA f(ld,nx,0:8), two lattices (9.66 GB,
far larger than the 129 MB L2, so no L2 flush is needed between steps).
Initial state: Taylor-Green vortex u0 = 0.05 (k = 2 pi / 8192) plus seeded
i.i.d. N(0, 1e-4^2) velocity noise, f at equilibrium.  A step is one
perform_lbm_step (one fused pull-stream + collide kernel) over the grid.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--n 8192] [--kind bgk|trt|rr] [--storage f64|f32dev|f16dev]
                    [--math fma|strict|hybrid]

Prints one JSON line (rank 0).  --impl reference times the reference's
algorithm on the host cores instead: the C restatement of the Fortran
(two passes per step, stream then collide, OpenMP over all host threads).
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
# dram__bytes_write.sum of one launch / cells), from profiles/.  None: no capture yet.
NCU_TRAFFIC_PER_CELL = {}
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


def workload_config(args) -> dict:
    return {"workload": f"plain single-grid bandwidth bench: D2Q9 {args.kind.upper()} tau={args.tau} "
                        f"{args.n}x{args.n} periodic, {args.storage} SoA two-lattice, TGV u0=0.05 + N(0,1e-4^2) noise",
            "grid": [args.n, args.n], "collision": args.kind, "tau": args.tau, "storage": args.storage,
            "math": args.math, "layout": "f(ld,nx,0:8) y-fastest, ld=pad16(ny)",
            "l2_policy": "inputs larger than L2 (two lattices of "
                         f"{2 * 9 * args.n * args.n * {'f64': 8, 'f32dev': 4, 'f16dev': 2}[args.storage] / 1e9:.2f} GB"
                         " vs 129 MB L2); no flush",
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU"}


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
    ap.add_argument("--math", default="fma", choices=["fma", "strict", "hybrid"])
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU-baseline sample length")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

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
    ms_t = torch.tensor([ms], device="cuda")
    if world > 1:
        dist.all_reduce(ms_t, op=dist.ReduceOp.MAX)
    ms_max = float(ms_t.item())
    cells = n * n
    mlups = world * cells * args.steps / (ms_max * 1e-3) / 1e6

    # ---- end to end through the C ABI with host buffers -------------------------
    # One job as the reference's time loop runs it: pinned host f(ld,nx,0:8) ->
    # plbm_upload, K plbm_perform_lbm_step(grid,1) calls, plbm_update_macros to
    # pinned host rho/ux/uy.  Copies are inside the timed region.
    ld = g.ld
    host_f = torch.empty((9, n, ld), dtype=torch.float64, pin_memory=True).numpy()
    host_f[...] = g.download(g.iold)
    host_m = [torch.empty((n, n), dtype=torch.float64, pin_memory=True).numpy() for _ in range(3)]
    lib = _lib.load()
    h = g.handle
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    _lib.check(lib.plbm_upload(h, host_f.ctypes.data, g.iold))
    for _ in range(args.steps):
        _lib.check(lib.plbm_perform_lbm_step(h, 1))
    _lib.check(lib.plbm_update_macros(h, *[m.ctypes.data for m in host_m]))
    torch.cuda.synchronize()
    e2e_s = time.perf_counter() - t0
    barrier()
    e2e_t = torch.tensor([e2e_s], device="cuda")
    if world > 1:
        dist.all_reduce(e2e_t, op=dist.ReduceOp.MAX)
    e2e_mlups = world * cells * args.steps / float(e2e_t.item()) / 1e6
    h2d = 9 * n * ld * 8
    d2h = 3 * n * n * 8
    g.close()

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
        "dtype": {"f64": "f64", "f32dev": "f32", "f16dev": "f16"}[args.storage] ,
        "data": "synthetic (seeded TGV + noise, no dataset)",
        "config": workload_config(args),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic * cells if traffic else None,
                     "peak_source": f"{peak_kind} hbm_gbs", "algorithmic_bytes_per_cell": BYTES_PER_CELL[args.storage]},
        "e2e": {"value": e2e_mlups, "unit": "MLUPS", "h2d_bytes_per_step": h2d / args.steps,
                "d2h_bytes_per_step": d2h / args.steps,
                "job": "plbm_upload(pinned f) + K x plbm_perform_lbm_step(1) + plbm_update_macros(pinned)"},
        "gpu_launches": args.steps,
        "clocks": clocks,
    }
    if not args.no_cpu_baseline:
        # bounded sample of the same workload: estimate one step, then size the run
        from oracle import oracle as O
        one = cpu_reference_run(n, args.kind, omega, 1, 1, fields)
        steps = max(1, min(50, int(args.cpu_seconds / max(one["seconds"], 1e-3))))
        r = cpu_reference_run(n, args.kind, omega, steps, 0, fields)
        line["cpu_baseline"] = {
            "value": r["mlups"], "unit": "MLUPS", "cores": r["threads"], "kind": "port",
            "sample": f"{n}x{n} {args.kind.upper()} binary64, {steps} steps (two passes each) of the C "
                      f"restatement, {r['threads']} OpenMP threads on {cpu_model()}"}
        del O
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
