"""The one-kernel StandardForm path (std_compact_kernel): StandardForm on
elements with at most 32 volume, facet and modal nodes runs one kernel per
residual (and per Runge-Kutta stage, the stage update applied by the same
kernel), the facet traces R V u evaluated from the element's and its
neighbours' modal coefficients.

Checked against the oracle at the parity tolerance (rel2 <= max(1e-12,
4 x the oracle's own round-off floor)) and against the two-phase kernels on
the same handle; Runge-Kutta trajectories of both schemes against the
oracle's; bitwise run-to-run; conservation of the advection residual (the
two traces of a shared facet node are bitwise equal, so the interface fluxes
cancel); the path's scope and switch."""
import numpy as np
import pytest

import cases
from oracle.oracle import Oracle, rel2, roundoff_floor

pytestmark = pytest.mark.gpu

# StandardForm cases whose elements fit one warp (triangles up to p = 4,
# tensor-product and multidimensional, modal and nodal, advection and Euler)
ONE_KERNEL = ["adv_tri_modal", "adv_tri_nodal", "adv_tri_central", "euler_tri_std", "multi_adv_tri",
              "multi_adv_tri_nodal", "multi_tri_std"]
# outside its scope: flux differencing, tets with 64 volume nodes
TWO_PHASE = ["adv_tri_fd", "vortex_tri_modal", "adv_tet_modal", "euler_tet_std"]


@pytest.mark.parametrize("name", ONE_KERNEL + TWO_PHASE)
def test_path_selected_where_it_applies(gpu_lib, pkg, name):
    host, _ = cases.make(name)
    G = pkg.GB300Solver(host)
    abi = pkg.abi
    if name in ONE_KERNEL:
        assert G.kernel_path() == abi.SSE_PATH_ONE_KERNEL
        G.set_kernel_path(abi.SSE_PATH_TWO_PHASE)
        assert G.kernel_path() == abi.SSE_PATH_TWO_PHASE
        G.set_kernel_path(abi.SSE_PATH_ONE_KERNEL)
        assert G.kernel_path() == abi.SSE_PATH_ONE_KERNEL
    else:
        assert G.kernel_path() == abi.SSE_PATH_TWO_PHASE
        with pytest.raises(pkg.SSEError) as e:
            G.set_kernel_path(abi.SSE_PATH_ONE_KERNEL)
        assert e.value.code == abi.SSE_ERR_UNSUPPORTED
        assert G.kernel_path() == abi.SSE_PATH_TWO_PHASE


@pytest.mark.parametrize("name", ONE_KERNEL)
def test_residual_matches_oracle_and_two_phase(gpu_lib, pkg, name):
    import torch
    host, u = cases.make(name)
    G = pkg.GB300Solver(host)
    got = G.residual(u)
    want = Oracle(host).residual(u)
    bound = max(1e-12, 4.0 * roundoff_floor(host, u))
    assert rel2(got, want) <= bound, rel2(got, want)
    G.set_kernel_path(pkg.abi.SSE_PATH_TWO_PHASE)
    two = G.residual(u)
    assert rel2(two, want) <= bound
    assert rel2(got, two) <= bound
    G.set_kernel_path(pkg.abi.SSE_PATH_ONE_KERNEL)
    # device buffers, bitwise run to run and equal to the host-buffer call
    ud = torch.from_numpy(u).cuda()
    a, b = torch.empty_like(ud), torch.empty_like(ud)
    G.residual(ud, a)
    G.residual(ud, b)
    torch.cuda.synchronize()
    assert torch.equal(a, b)
    assert np.array_equal(a.cpu().numpy(), got)


@pytest.mark.parametrize("name", ["adv_tri_modal", "euler_tri_std", "multi_tri_std"])
@pytest.mark.parametrize("scheme", [0, 1])
def test_stages_match_oracle(gpu_lib, pkg, name, scheme):
    """Five CK2N54 stages (ping-pong buffers, copied back) or four RK4 stages
    (two alternating stage inputs) per step, each one launch."""
    host, u = cases.make(name)
    G = pkg.GB300Solver(host)
    assert G.kernel_path() == pkg.abi.SSE_PATH_ONE_KERNEL
    dt = 1.0e-3
    for steps in (1, 4):           # a direct step and a replayed (graph) step
        ug = u.copy()
        t = G.rk_steps(ug, steps, dt, scheme)
        assert abs(t - steps * dt) < 1e-15
        uo = Oracle(host).rk_steps(u, steps, dt, scheme)
        assert rel2(ug, uo) <= 1e-12, (steps, rel2(ug, uo))
        G.set_kernel_path(pkg.abi.SSE_PATH_TWO_PHASE)
        u2 = u.copy()
        G.rk_steps(u2, steps, dt, scheme)
        G.set_kernel_path(pkg.abi.SSE_PATH_ONE_KERNEL)
        assert rel2(ug, u2) <= 1e-12


def test_advection_interface_fluxes_cancel(gpu_lib, pkg):
    """The integral of the advection residual over a periodic mesh is zero:
    the two traces of each shared facet node are the same arithmetic on the
    same coefficients, so the Lax-Friedrichs fluxes cancel pairwise."""
    host, u = cases.make("adv_tri_modal")
    G = pkg.GB300Solver(host)
    r = G.residual(u)
    out = G.conservation_residual(u, r)
    scale = float(np.abs(r).max())
    assert abs(out[0]) < 1e-12 * scale * host.N_e


def test_phase_timings_report_one_kernel(gpu_lib, pkg):
    import torch
    host, u = cases.make("adv_tri_modal")
    G = pkg.GB300Solver(host)
    t = G.phase_timings(torch.from_numpy(u).cuda(), 3)
    assert t[0] == 0.0 and t[1] > 0.0
    G.set_kernel_path(pkg.abi.SSE_PATH_TWO_PHASE)
    t = G.phase_timings(torch.from_numpy(u).cuda(), 3)
    assert t[0] > 0.0 and t[1] > 0.0


def test_residual_written_over_its_input(gpu_lib, pkg):
    """dudt aliasing u: the neighbours' traces read u, so that call takes the
    two-phase kernels and still returns R(u)."""
    import torch
    host, u = cases.make("adv_tri_modal")
    G = pkg.GB300Solver(host)
    want = G.residual(u)
    ud = torch.from_numpy(u.copy()).cuda()
    G.residual(ud, ud)
    torch.cuda.synchronize()
    assert rel2(ud.cpu().numpy(), want) <= 1e-13
