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
        # each call restarts the compensation of the stage accumulation
        assert float(torch.linalg.norm(a - b) / torch.linalg.norm(b)) < 1e-13
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
        assert float(torch.linalg.norm(c - d) / torch.linalg.norm(d)) < 1e-13
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
