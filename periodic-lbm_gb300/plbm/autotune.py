"""Autotuner of the batched stepper's schedule (tile shapes and CTA layout).

The search space is the ``plbm_batch_schedule``: threads per CTA, resident
CTAs per SM, persistent (one cooperative launch) or one launch per step, and
the tile height ty for each of the five ny buckets.  The search times short
runs of the actual batch with CUDA events:

1. for threads in {128, 256, 512} x persistent in {1, 0} with the default ty
   table, keep the fastest (and the fastest of the other mode);
2. coordinate descent over the ty of each bucket that holds grids;
3. resident CTAs per SM in {occupancy maximum, 1, 2, 4};
4. the winner against the best schedule of the other mode (persistent or per
   step) on longer runs (final_steps): the persistent launch pays its setup
   once per run, which short trials overweight.

The winner is cached in a JSON file keyed by the batch signature (grid sizes,
kinds, storage, collision arithmetic, device), so later runs of the same batch reuse it.  The
schedule changes only the work decomposition: results are bit-identical for
every schedule.
"""
from __future__ import annotations

import hashlib
import json
import os
from pathlib import Path

from .batched import BUCKETS, BatchedGrids, Schedule

CACHE = Path(os.environ.get("PLBM_AUTOTUNE_CACHE", Path(__file__).resolve().parent / "autotune_cache.json"))
BUCKET_EDGES = (48, 96, 192, 384)


def bucket_of(ny: int) -> int:
    for i, e in enumerate(BUCKET_EDGES):
        if ny <= e:
            return i
    return BUCKETS - 1


def signature(batch: BatchedGrids, device: str) -> str:
    h = hashlib.sha256()
    for s in batch.specs:
        h.update(f"{s.nx},{s.ny},{s.kind};".encode())
    h.update(f"{batch.storage}|{getattr(batch, 'math', 'fma')}|{device}".encode())
    return h.hexdigest()[:24]


def _time(batch: BatchedGrids, steps: int, reps: int) -> float:
    import torch
    stream = torch.cuda.Stream()
    batch.set_stream(stream.cuda_stream)
    batch.run(2)
    batch.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        batch.run(steps)
        e1.record(stream)
        batch.synchronize()
        best = min(best, e0.elapsed_time(e1) / steps)
    batch.set_stream(None)
    return best


def tune(batch: BatchedGrids, steps: int = 10, reps: int = 2, use_cache: bool = True,
         verbose: bool = False, final_steps: int = 50) -> tuple[Schedule, dict]:
    """Search a schedule for `batch`; sets it and returns (schedule, report)."""
    import torch
    dev = torch.cuda.get_device_name()
    key = signature(batch, dev)
    cache = {}
    if CACHE.exists():
        try:
            cache = json.loads(CACHE.read_text())
        except Exception:
            cache = {}
    if use_cache and key in cache:
        s = Schedule.from_dict(cache[key]["schedule"])
        batch.schedule = s
        return s, dict(cache[key], cached=True)

    trials = []

    def trial(s: Schedule) -> float:
        batch.schedule = s
        ms = _time(batch, steps, reps)
        trials.append((s.as_dict(), ms))
        if verbose:
            print(f"  {s.as_dict()} -> {ms:.4f} ms/step")
        return ms

    base = batch.schedule
    best, best_ms = None, float("inf")
    by_mode = {}  # persistent -> (schedule, ms) of stage 1
    for threads in (128, 256, 512):
        for persistent in (1, 0):
            s = Schedule.from_dict(base.as_dict())
            s.threads, s.persistent, s.ctas_per_sm = threads, persistent, 0
            for i in range(BUCKETS):
                s.ty[i] = min(s.ty[i], threads)
            ms = trial(s)
            if ms < best_ms:
                best, best_ms = s, ms
            if persistent not in by_mode or ms < by_mode[persistent][1]:
                by_mode[persistent] = (s, ms)
    used = sorted({bucket_of(sp.ny) for sp in batch.specs})
    for b in used:
        for ty in (32, 64, 128, 256, 512):
            if ty > best.threads or ty == best.ty[b]:
                continue
            s = Schedule.from_dict(best.as_dict())
            s.ty[b] = ty
            ms = trial(s)
            if ms < best_ms:
                best, best_ms = s, ms
    for cps in (1, 2, 4):
        s = Schedule.from_dict(best.as_dict())
        s.ctas_per_sm = cps
        ms = trial(s)
        if ms < best_ms:
            best, best_ms = s, ms
    other = by_mode.get(1 - best.persistent)
    if other is not None and final_steps > steps:
        batch.schedule = best
        ms_best = _time(batch, final_steps, 1)
        batch.schedule = other[0]
        ms_other = _time(batch, final_steps, 1)
        trials.append((other[0].as_dict(), ms_other))
        if verbose:
            print(f"  final: {best.as_dict()} -> {ms_best:.4f}, {other[0].as_dict()} -> {ms_other:.4f} ms/step")
        if ms_other < ms_best:
            best, best_ms = other[0], ms_other
        else:
            best_ms = ms_best
    batch.schedule = best
    report = {"schedule": best.as_dict(), "ms_per_step": best_ms, "trials": len(trials), "device": dev}
    cache[key] = report
    try:
        CACHE.write_text(json.dumps(cache, indent=1))
    except OSError:
        pass
    return best, dict(report, cached=False)
