"""GPU tests of the batched stepper (plbm_batch_*): every grid of a batch
advances exactly as a single lattice_grid does, for every schedule, launch
mode and graph replay."""
import math

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu

SPECS = [(17, 13, "bgk", 1.25), (32, 48, "trt", 1.6), (64, 20, "bgk", 1.9), (100, 37, "trt", 0.8),
         (33, 33, "bgk", 1.5), (256, 64, "trt", 1.1), (9, 300, "bgk", 1.7)]


def make_batch(storage="f64"):
    from plbm.batched import BatchedGrids, GridSpec
    specs = [GridSpec(nx, ny, k, om, 0.25) for nx, ny, k, om in SPECS]
    b = BatchedGrids(specs, storage)
    fields = []
    rng = np.random.default_rng(4)
    for i, (nx, ny, _, _) in enumerate(SPECS):
        x = (np.arange(nx) + 0.5)[:, None] * 2 * np.pi / nx
        y = (np.arange(ny) + 0.5)[None, :] * 2 * np.pi / ny
        ux = 0.04 * np.cos(x) * np.sin(2 * y) + 1e-4 * rng.standard_normal((nx, ny))
        uy = -0.03 * np.sin(x) * np.cos(y) + 1e-4 * rng.standard_normal((nx, ny))
        rho = 1.0 + 1e-3 * rng.standard_normal((nx, ny))
        b.set_equilibrium(i, rho, ux, uy)
        fields.append((rho, ux, uy))
    return b, fields


def oracle_grid(i, fields, steps):
    nx, ny, kind, om = SPECS[i]
    f2 = np.stack([np.zeros((9, nx, O.pad16(ny))), O.set_pdf_to_equilibrium(*fields[i])])
    iold, _ = O.perform_lbm_step(f2, ny, 2, 1, {"bgk": O.BGK, "trt": O.TRT}[kind], om, 0.25, steps)
    return f2[iold - 1]


def relinf(a, b):
    return float(np.max(np.abs(a - b)) / np.max(np.abs(b)))


def test_batched_f64_matches_oracle_per_grid(gpu_lib):
    b, fields = make_batch()
    b.run(3)
    b.run(8)  # odd + even step counts: lattice parity is tracked
    b.synchronize()
    assert b.steps == 11
    for i, (nx, ny, _, _) in enumerate(SPECS):
        got = b.download(i)
        ref = oracle_grid(i, fields, 11)
        for a, c in zip(O.update_macros(got, ny), O.update_macros(ref, ny)):
            assert relinf(a, c) <= 1e-12
    b.close()


def _states(b):
    return [b.download(i) for i in range(len(SPECS))]


@pytest.mark.parametrize("threads,persistent,ty", [(128, 1, [32, 32, 32, 32, 32]), (256, 0, [32, 64, 128, 256, 256]),
                                                   (512, 1, [64, 128, 256, 512, 512]), (64, 0, [32, 64, 64, 64, 64])])
def test_schedule_does_not_change_results(gpu_lib, threads, persistent, ty):
    from plbm.batched import Schedule
    ref, _ = make_batch()
    ref.run(6)
    want = _states(ref)
    ref.close()
    b, _ = make_batch()
    b.schedule = Schedule.from_dict({"threads": threads, "ctas_per_sm": 0, "persistent": persistent, "ty": ty})
    b.run(6)
    got = _states(b)
    for a, c in zip(got, want):
        assert np.array_equal(a, c)
    b.close()


def test_graph_replay_equals_direct_run(gpu_lib):
    a, _ = make_batch()
    a.run(10)
    want = _states(a)
    a.close()
    b, _ = make_batch()
    b.capture(5)  # graph for parity 0 (5 steps)
    b.launch_graph()  # steps 0..4, now parity 1
    b.capture(5)
    b.launch_graph()  # steps 5..9
    b.synchronize()
    assert b.steps == 10
    got = _states(b)
    for x, y in zip(got, want):
        assert np.array_equal(x, y)
    b.close()


def test_batched_f32dev_close_to_f64(gpu_lib):
    a, _ = make_batch("f64")
    d, _ = make_batch("f32dev")
    a.run(50)
    d.run(50)
    for i, (nx, ny, _, _) in enumerate(SPECS):
        _, u, v = a.macros(i)
        _, ud, vd = d.macros(i)
        err = math.sqrt(np.sum((ud - u) ** 2 + (vd - v) ** 2) / np.sum(u ** 2 + v ** 2))
        assert err < 1e-4
    a.close()
    d.close()


def test_autotuner_picks_a_schedule_and_keeps_results(gpu_lib, tmp_path, monkeypatch):
    from plbm import autotune
    monkeypatch.setattr(autotune, "CACHE", tmp_path / "cache.json")
    b, _ = make_batch()
    ref, _ = make_batch()
    s, rep = autotune.tune(b, steps=3, reps=1)
    assert rep["trials"] > 6 and not rep["cached"]
    s2, rep2 = autotune.tune(b, steps=3, reps=1)
    assert rep2["cached"] and s2.as_dict() == s.as_dict()
    # tuning ran steps; compare from a fresh state
    b.close()
    b, _ = make_batch()
    b.schedule = s
    b.run(4)
    ref.run(4)
    for x, y in zip(_states(b), _states(ref)):
        assert np.array_equal(x, y)
    b.close()
    ref.close()


def test_batch_input_errors(gpu_lib):
    from plbm import PlbmError
    from plbm.batched import BatchedGrids, GridSpec, Schedule
    with pytest.raises(PlbmError):
        BatchedGrids([GridSpec(8, 8, "rr", 1.2)])
    b = BatchedGrids([GridSpec(8, 8, "bgk", 1.2)])
    with pytest.raises(PlbmError):
        b.schedule = Schedule.from_dict({"threads": 100, "ctas_per_sm": 0, "persistent": 1, "ty": [32] * 5})
    with pytest.raises(PlbmError):
        b.launch_graph()  # nothing captured
    b.close()


def make_batch_math(storage, math):
    b, fields = make_batch(storage)
    b.set_math(math)
    return b, fields


def test_batched_hybrid_matches_oracle_per_grid(gpu_lib):
    """Hybrid binary64 arithmetic on the BGK grids (TRT grids stay FMA):
    every grid within 1e-12 of the oracle, and independent of the schedule."""
    from plbm.batched import Schedule
    b, fields = make_batch_math("f64", "hybrid")
    b.run(7)
    b.run(6)
    for i, (nx, ny, _, _) in enumerate(SPECS):
        got = b.download(i)
        ref = oracle_grid(i, fields, 13)
        for a, c in zip(O.update_macros(got, ny), O.update_macros(ref, ny)):
            assert relinf(a, c) <= 1e-12
    want = _states(b)
    b.close()
    p, _ = make_batch_math("f64", "hybrid")
    p.schedule = Schedule.from_dict({"threads": 128, "ctas_per_sm": 0, "persistent": 0, "ty": [32] * 5})
    p.run(13)
    for x, y in zip(_states(p), want):
        assert np.array_equal(x, y)
    p.close()


@pytest.mark.parametrize("kind", ["bgk", "trt"])
def test_batched_hybrid_falls_back_outside_range(gpu_lib, kind):
    """A grid holding populations past the hybrid limits (f_0 >= 2) takes the
    FMA binary64 operator in those cells: the result equals the FMA batch's
    to 1e-12."""
    from plbm.batched import BatchedGrids, GridSpec
    specs = [GridSpec(16, 32, kind, 1.3)]
    rng = np.random.default_rng(9)
    rho = 5.0 + 0.01 * rng.standard_normal((16, 32))  # f_0 = 4/9 rho > 2
    ux = 0.02 * rng.standard_normal((16, 32))
    uy = 0.02 * rng.standard_normal((16, 32))
    outs = []
    for m in ("fma", "hybrid"):
        b = BatchedGrids(specs, "f64", math=m)
        b.set_equilibrium(0, rho, ux, uy)
        b.run(5)
        outs.append(b.download(0))
        b.close()
    assert relinf(outs[1], outs[0]) <= 1e-12


def test_batched_hybrid_rejected_for_f32dev(gpu_lib):
    from plbm import PlbmError
    b, _ = make_batch("f32dev")
    with pytest.raises(PlbmError):
        b.set_math("hybrid")
    b.close()


def test_persistent_barrier_wait_runs_out_and_the_context_survives(gpu_lib):
    """Bounded-wait failure path: the injected run's grid barrier can never
    complete; every CTA gives up after its bounded wait, the host reads
    PLBM_E_TIMEOUT, and the same device then runs a batch correctly."""
    from plbm import PlbmError
    from plbm.batched import Schedule
    b, _ = make_batch()
    b.schedule = Schedule.from_dict({"threads": 128, "ctas_per_sm": 0, "persistent": 1, "ty": [32] * 5})
    b.inject_stall()
    b.run(3)
    with pytest.raises(PlbmError) as e:
        b.synchronize()
    assert e.value.code == -5
    b.close()
    ok, fields = make_batch()
    ok.schedule = Schedule.from_dict({"threads": 128, "ctas_per_sm": 0, "persistent": 1, "ty": [32] * 5})
    ok.run(4)
    ok.synchronize()
    for i, (nx, ny, _, _) in enumerate(SPECS):
        for a, c in zip(O.update_macros(ok.download(i), ny), O.update_macros(oracle_grid(i, fields, 4), ny)):
            assert relinf(a, c) <= 1e-12
    ok.close()
