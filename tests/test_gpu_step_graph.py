"""sse_rk_steps replays one captured Runge-Kutta step (a CUDA graph) when it
advances several steps; the result must be bitwise the one of the same
steps launched one call at a time, for both schemes and both precisions,
and a changed step size or state buffer must be honoured."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name,scheme,mixed", [("vortex_tri_modal", 0, False), ("vortex_tri_modal", 1, False),
                                               ("tgv_tet_modal", 0, False), ("tgv_tet_modal", 0, True),
                                               ("adv_tri_modal", 1, False)])
def test_replayed_steps_match_single_steps(name, scheme, mixed, gpu_lib, pkg):
    import torch
    host, u0 = cases.make(name)
    G = pkg.GB300Solver(host)
    if mixed:
        G.set_precision(pkg.abi.SSE_MIXED)
    dt = 1e-3
    a = torch.from_numpy(u0.copy()).cuda()
    G.rk_steps(a, 6, dt, scheme)
    b = torch.from_numpy(u0.copy()).cuda()
    for _ in range(6):
        G.rk_steps(b, 1, dt, scheme)
    torch.cuda.synchronize()
    if mixed:
        # each call restarts the compensation of the stage accumulation: the
        # states then differ in their last bits, which can flip FP32
        # roundings of the perturbations (far inside the form's 1e-6 budget)
        assert float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) < 1e-8
    else:
        assert torch.equal(a, b)
    # a new step size and a new buffer are captured afresh
    c = torch.from_numpy(u0.copy()).cuda()
    G.rk_steps(c, 3, 2 * dt, scheme)
    d = torch.from_numpy(u0.copy()).cuda()
    for _ in range(3):
        G.rk_steps(d, 1, 2 * dt, scheme)
    torch.cuda.synchronize()
    if mixed:
        assert float(torch.linalg.norm(c - d) / torch.linalg.norm(d)) < 1e-8
    else:
        assert torch.equal(c, d)
    assert not torch.equal(c, a)
    # host buffers go through the handle's staging buffer and the same graph
    h = u0.copy()
    G.rk_steps(h, 6, dt, scheme)
    assert np.array_equal(h, a.cpu().numpy()) or mixed


@pytest.mark.parametrize("scheme,device", [(0, True), (1, False)])
def test_snapshot_hook(scheme, device, gpu_lib, pkg):
    """sse_rk_steps_snapshots (the save_callback hook): the states after every
    k-th step and their residuals, bitwise those of stepping k at a time."""
    import torch
    host, u0 = cases.make("vortex_tri_modal")
    G = pkg.GB300Solver(host)
    dt = 1e-3
    u = torch.from_numpy(u0.copy()).cuda() if device else u0.copy()
    t, snaps, res = G.rk_steps_snapshots(u, 7, dt, every=3, scheme=scheme, with_residuals=True)
    assert t == pytest.approx(7 * dt)
    assert snaps.shape[0] == 2 and res.shape[0] == 2
    if device:
        torch.cuda.synchronize()
        snaps, res, u = snaps.cpu().numpy(), res.cpu().numpy(), u.cpu().numpy()
    w = u0.copy()
    for i in range(2):
        G.rk_steps(w, 3, dt, scheme)
        assert np.array_equal(snaps[i], w)
        assert np.array_equal(res[i], G.residual(w))
    G.rk_steps(w, 1, dt, scheme)
    assert np.array_equal(u, w)


# Carpenter & Kennedy (1994) five-stage fourth-order 2N-storage coefficients
_CK_A = (0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
         -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0)
_CK_B = (1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
         1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
         2277821191437.0 / 14882151754819.0)


@pytest.mark.parametrize("name,mixed", [("vortex_tri_modal", False), ("tgv_tet_modal", False),
                                        ("vortex_tri_modal", True), ("tgv_tet_modal", True)])
def test_ck_steps_match_explicit_stages(name, mixed, gpu_lib, pkg):
    """sse_rk_steps' CarpenterKennedy2N54 steps (residual kernels and the
    stage-update kernel replayed as one captured step) equal the explicit
    low-storage recurrence tmp = a tmp + dt r, u += b tmp on residuals
    evaluated one call at a time, up to the rounding of the stage arithmetic
    (contracted multiply-adds, compensated summation in the mixed form,
    whose FP32 perturbations can round differently once the states differ
    in their last bits)."""
    import torch
    host, u0 = cases.make(name)
    G = pkg.GB300Solver(host)
    if mixed:
        G.set_precision(pkg.abi.SSE_MIXED)
    dt = 1e-3
    fused = torch.from_numpy(u0.copy()).cuda()
    G.rk_steps(fused, 2, dt, 0)
    u = torch.from_numpy(u0.copy()).cuda()
    tmp = torch.zeros_like(u)
    for _ in range(2):
        for a, b in zip(_CK_A, _CK_B):
            r = G.residual(u)
            tmp = a * tmp + dt * r
            u = u + b * tmp
    torch.cuda.synchronize()
    change = float(torch.linalg.norm(u - torch.from_numpy(u0).cuda()))
    assert change > 0
    assert float(torch.linalg.norm(fused - u)) <= (1e-5 if mixed else 1e-11) * change
