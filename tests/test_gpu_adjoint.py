"""GPU tests of the discrete adjoint and its torch.autograd.Function:
against the FP64 CPU adjoint, against central finite differences of the
binary64 model, invariance under the checkpoint interval, and the binary32
deviation-storage adjoint against the binary64 one."""
import math

import numpy as np
import pytest

from oracle import oracle as O

pytestmark = pytest.mark.gpu


def fields(nx, ny, seed=3, amp=0.01):
    from plbm import cases
    ux, uy = cases.divergence_free_modes(max(nx, ny), nmodes=8, kmax=4, amp=amp, seed=seed)
    return np.ascontiguousarray(ux[:nx, :ny]), np.ascontiguousarray(uy[:nx, :ny])


def test_gpu_adjoint_matches_cpu_adjoint(gpu_lib):
    import torch
    from plbm.autograd import Adjoint
    nx, ny, steps, omega = 40, 28, 60, 1.4
    ux0, uy0 = fields(nx, ny)
    tx, ty = fields(nx, ny, seed=5)
    (uT, vT) = O.forward_bgk(ux0, uy0, omega, steps)
    _, (gx, gy), gom = O.adjoint_bgk(ux0, uy0, omega, steps, uT - tx, vT - ty)
    a = Adjoint(nx, ny, steps, checkpoint_every=7, storage="f64")
    u0 = torch.tensor(np.stack([ux0, uy0]), device="cuda")
    uTg = a.forward(u0, omega)
    got_uT = uTg.cpu().numpy()
    assert np.max(np.abs(got_uT[0] - uT)) <= 1e-12 * np.max(np.abs(uT))
    G = uTg - torch.tensor(np.stack([tx, ty]), device="cuda")
    g0, dom = a.backward(G)
    g0 = g0.cpu().numpy()
    scale = np.max(np.abs(np.stack([gx, gy])))
    assert np.max(np.abs(g0[0] - gx)) <= 1e-9 * scale
    assert np.max(np.abs(g0[1] - gy)) <= 1e-9 * scale
    assert abs(dom - gom) <= 1e-9 * abs(gom)
    a.close()


def test_checkpoint_interval_does_not_change_gradients(gpu_lib):
    import torch
    from plbm.autograd import Adjoint
    nx, ny, steps = 33, 20, 50
    ux0, uy0 = fields(nx, ny)
    u0 = torch.tensor(np.stack([ux0, uy0]), device="cuda")
    res = []
    for k in (1, 7, 50, 13):
        a = Adjoint(nx, ny, steps, checkpoint_every=k)
        uT = a.forward(u0, 1.2)
        g, dom = a.backward(uT)  # loss 0.5 |u_T|^2
        res.append((g.cpu().numpy(), dom))
        a.close()
    for g, dom in res[1:]:
        assert np.array_equal(g, res[0][0]) and dom == res[0][1]


@pytest.mark.parametrize("storage", ["f64", "f32dev"])
def test_one_segment_buffer_schedule_gives_the_same_gradients(gpu_lib, monkeypatch, storage):
    """The reverse sweep recomputes the next segment on a second stream into a
    second buffer; when that buffer does not fit it falls back to one buffer,
    each recomputation after the previous sweep.  Both schedules run the same
    kernels on the same data in the same order on the caller's stream: the
    gradients are bit-identical, the fallback holds K lattices fewer."""
    import torch
    from plbm.autograd import Adjoint
    nx, ny, steps, k = 40, 24, 61, 9
    ux0, uy0 = fields(nx, ny)
    u0 = torch.tensor(np.stack([ux0, uy0]), device="cuda")
    res, mem = [], []
    for one in ("0", "1"):
        monkeypatch.setenv("PLBM_ADJOINT_ONE_SEGMENT", one)
        a = Adjoint(nx, ny, steps, checkpoint_every=k, storage=storage)
        uT = a.forward(u0, 1.3)
        g, dom = a.backward(uT)
        res.append((g.cpu().numpy(), dom))
        mem.append(a.memory_bytes())
        a.close()
    assert np.array_equal(res[0][0], res[1][0]) and res[0][1] == res[1][1]
    lat = 9 * nx * (ny + (-ny) % 16) * (8 if storage == "f64" else 4)
    assert mem[0] - mem[1] == k * lat


def test_autograd_against_central_differences(gpu_lib):
    """dL/du0 and dL/dtau of L = 1/2 |u_T - u*|^2 by the adjoint vs central
    differences (h = 1e-4 relative) of the binary64 forward model."""
    import torch
    from plbm.autograd import lbm_final_velocity, velocity_misfit
    nx = ny = 48
    steps = 120
    ux0, uy0 = fields(nx, ny, seed=1)
    tx, ty = fields(nx, ny, seed=2)
    u0 = torch.tensor(np.stack([ux0, uy0]), device="cuda", requires_grad=True)
    tau = torch.tensor(0.8, dtype=torch.float64, device="cuda", requires_grad=True)
    target = torch.tensor(np.stack([tx, ty]), device="cuda")
    L = velocity_misfit(u0, tau, target, steps, checkpoint_every=11)
    L.backward()
    gu = u0.grad.cpu().numpy()

    def loss(u, t):
        with torch.no_grad():
            return float(0.5 * torch.sum((lbm_final_velocity(u, t, steps) - target) ** 2))

    rng = np.random.default_rng(0)
    scale = np.max(np.abs(gu))
    for _ in range(8):
        a, i, j = int(rng.integers(2)), int(rng.integers(nx)), int(rng.integers(ny))
        h = 1e-4 * max(abs(u0[a, i, j].item()), 1e-3)
        up = u0.detach().clone()
        um = u0.detach().clone()
        up[a, i, j] += h
        um[a, i, j] -= h
        fd = (loss(up, 0.8) - loss(um, 0.8)) / (2 * h)
        assert abs(fd - gu[a, i, j]) <= 1e-5 * scale, (a, i, j, fd, gu[a, i, j])
    h = 1e-4 * 0.8
    fd_tau = (loss(u0.detach(), 0.8 + h) - loss(u0.detach(), 0.8 - h)) / (2 * h)
    assert abs(fd_tau - float(tau.grad)) <= 1e-5 * abs(fd_tau)


def test_f32_adjoint_close_to_f64_adjoint(gpu_lib):
    import torch
    from plbm.autograd import Adjoint
    nx, ny, steps = 64, 64, 100
    ux0, uy0 = fields(nx, ny, seed=7)
    tx, ty = fields(nx, ny, seed=8)
    u0 = torch.tensor(np.stack([ux0, uy0]), device="cuda")
    tgt = torch.tensor(np.stack([tx, ty]), device="cuda")
    out = {}
    for st in ("f64", "f32dev"):
        a = Adjoint(nx, ny, steps, checkpoint_every=10, storage=st)
        uT = a.forward(u0, 1.25)
        out[st] = a.backward(uT - tgt)
        a.close()
    g64, d64 = out["f64"]
    g32, d32 = out["f32dev"]
    rel = float(torch.linalg.norm(g32 - g64) / torch.linalg.norm(g64))
    print(f"f32dev vs f64 adjoint: dL/du0 relative L2 {rel:.2e}, dL/domega rel {abs(d32 - d64) / abs(d64):.2e}")
    assert rel < 1e-3
    assert abs(d32 - d64) <= 1e-3 * abs(d64)


def test_compensated_reverse_step_is_closer_to_binary64(gpu_lib):
    """plbm_adjoint_set_math(PLBM_MATH_HYBRID) on binary32 storage: the
    compensated reverse step's gradients lie closer to the binary64 adjoint's
    than the plain binary32 step's, and it is refused for binary64 storage."""
    import torch
    from plbm import PlbmError
    from plbm.autograd import Adjoint
    nx, ny, steps = 64, 64, 300
    ux0, uy0 = fields(nx, ny, seed=7)
    tx, ty = fields(nx, ny, seed=8)
    u0 = torch.tensor(np.stack([ux0, uy0]), device="cuda")
    tgt = torch.tensor(np.stack([tx, ty]), device="cuda")
    out = {}
    for st, m in (("f64", "fma"), ("f32dev", "fma"), ("f32dev", "hybrid")):
        a = Adjoint(nx, ny, steps, checkpoint_every=17, storage=st, math=m)
        uT = a.forward(u0, 1.25)
        out[st, m] = a.backward(uT - tgt)
        a.close()
    g64, d64 = out["f64", "fma"]
    err = {}
    for m in ("fma", "hybrid"):
        g, d = out["f32dev", m]
        err[m] = (float(torch.linalg.norm(g - g64) / torch.linalg.norm(g64)), abs(d - d64) / abs(d64))
    print(f"f32dev vs f64 adjoint: plain {err['fma']}, compensated {err['hybrid']}")
    assert err["hybrid"][0] < err["fma"][0] and err["hybrid"][1] < err["fma"][1]
    with pytest.raises(PlbmError):
        Adjoint(16, 16, 10, storage="f64", math="hybrid")


def test_adjoint_errors(gpu_lib):
    from plbm import PlbmError
    from plbm.autograd import Adjoint
    import torch
    a = Adjoint(16, 16, 10)
    with pytest.raises(PlbmError):
        a.backward(torch.zeros((2, 16, 16), dtype=torch.float64, device="cuda"))  # no forward yet
    a.close()


def config5_problem(n=1024, seed_u=1, seed_t=2):
    """The adjoint inverse problem at full size: a divergence-free initial
    velocity of 16 Fourier modes |k| <= 8, amplitudes N(0, 0.01^2) (seed 1),
    the target from seed 2, tau = 0.8."""
    import torch
    from plbm import cases
    ux, uy = cases.divergence_free_modes(n, 16, 8, 0.01, seed=seed_u)
    tx, ty = cases.divergence_free_modes(n, 16, 8, 0.01, seed=seed_t)
    return (torch.tensor(np.stack([ux, uy]), device="cuda"), torch.tensor(np.stack([tx, ty]), device="cuda"))


def test_config5_gradient_against_central_differences_full_size(gpu_lib):
    """1024^2 D2Q9 BGK, T = 2000 steps, checkpoints every 45: dL/du0 and
    dL/dtau of L = 1/2 |u_T - u*|^2 from the binary64 discrete adjoint against
    central differences (h = 1e-4) of the binary64 forward model on 32 seeded
    random components of u0 and on tau, each within 1e-5 relative; then the
    binary32-storage model's adjoint gradient against the binary64 one: within
    5e-5 (dL/du0, norm-wise) and 1.5e-4 (dL/dtau) of it, and with the
    compensated reverse step within 1.5e-5 and 4e-5 (the bench records the
    figures)."""
    import torch
    from plbm.autograd import Adjoint
    n, T, K, tau, h = 1024, 2000, 45, 0.8, 1e-4
    u0, tgt = config5_problem(n)
    a = Adjoint(n, n, T, K, "f64")
    uT = a.forward(u0, 1.0 / tau)
    g, dom = a.backward(uT - tgt)
    gtau = -dom / tau ** 2
    g = g.cpu().numpy()

    def diff_loss(up, um, tp, tm):
        # L(+) - L(-) summed as 1/2 (a - b)(a + b - 2 t): no cancellation of the two totals
        Up, Um = a.forward(up, 1.0 / tp), a.forward(um, 1.0 / tm)
        return float(torch.sum(0.5 * (Up - Um) * (Up + Um - 2.0 * tgt)))

    rng = np.random.default_rng(2024)
    worst = 0.0
    for _ in range(32):
        c, i, j = int(rng.integers(2)), int(rng.integers(n)), int(rng.integers(n))
        up, um = u0.clone(), u0.clone()
        up[c, i, j] += h
        um[c, i, j] -= h
        fd = diff_loss(up, um, tau, tau) / (2 * h)
        rel = abs(fd - g[c, i, j]) / abs(g[c, i, j])
        worst = max(worst, rel)
        assert rel <= 1e-5, (c, i, j, fd, g[c, i, j], rel)
    fd_tau = diff_loss(u0, u0, tau + h, tau - h) / (2 * h)
    rel_tau = abs(fd_tau - gtau) / abs(gtau)
    print(f"config 5: worst dL/du0 component error {worst:.2e}, dL/dtau error {rel_tau:.2e}")
    assert rel_tau <= 1e-5, (fd_tau, gtau)
    a.close()
    b = Adjoint(n, n, T, K, "f32dev")
    uT32 = b.forward(u0, 1.0 / tau)
    g32, dom32 = b.backward(uT32 - tgt)
    b.close()
    g64 = torch.tensor(g, device="cuda")
    rel32 = float(torch.linalg.norm(g32 - g64) / torch.linalg.norm(g64))
    rel32_tau = abs(-dom32 / tau ** 2 - gtau) / abs(gtau)
    print(f"config 5: binary32-storage gradient vs binary64: dL/du0 {rel32:.2e}, dL/dtau {rel32_tau:.2e}")
    # measured 3.0e-5 and 8.0e-5 (both runs are deterministic: fixed-order sums)
    assert rel32 <= 5e-5 and rel32_tau <= 1.5e-4
    c = Adjoint(n, n, T, K, "f32dev", math="hybrid")
    uTc = c.forward(u0, 1.0 / tau)
    gc, domc = c.backward(uTc - tgt)
    c.close()
    relc = float(torch.linalg.norm(gc - g64) / torch.linalg.norm(g64))
    relc_tau = abs(-domc / tau ** 2 - gtau) / abs(gtau)
    print(f"config 5: compensated reverse step vs binary64: dL/du0 {relc:.2e}, dL/dtau {relc_tau:.2e}")
    # measured 9.4e-6 and 2.7e-5
    assert relc <= 1.5e-5 and relc_tau <= 4e-5
