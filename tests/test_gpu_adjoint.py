"""Discrete adjoint on the GPU (sse_residual_vjp, sse_rk_record /
sse_rk_adjoint) against the dual-number oracle: the dot-product identity
<lam, J v> = <J^T lam, v> to round-off, the full transposed Jacobian on a
small mesh, the adjoint Runge-Kutta sweep against the tangent of the whole
oracle trajectory, checkpoint-interval invariance, the mixed-form
recording, and central differences of an objective through the GPU
forward."""
import math

import numpy as np
import pytest

import cases
from oracle import oracle as O

pytestmark = pytest.mark.gpu

ADJ_NAMES = ["vortex_tri_modal", "vortex_tri_nodal", "vortex_tri_ec", "tgv_tet_modal", "tgv_tet_ec",
             "tgv_tet_nodal", "tgv_tet_p5", "tgv_tet_p2",
             # StandardForm: linear advection (LF / central, modal / nodal, Tri / Tet) and Euler
             "adv_tri_modal", "adv_tri_nodal", "adv_tri_central", "adv_tet_modal", "euler_tri_std",
             # FluxDifferencingForm with the conservative two-point flux
             "adv_tri_fd", "adv_tet_fd", "vortex_tri_cons2pt", "tgv_tet_cons2pt", "euler_tet_std",
             # multidimensional (dense V, D, R) approximations
             "multi_adv_tri", "multi_adv_tri_fd", "multi_tri", "multi_tri_nodal", "multi_tri_std",
             "multi_tet",
             # exact metrics (no free-stream preservation on curved tets)
             "tgv_tet_exact", "vortex_tri_exact"]


def _dot_rel(a, b, c, d):
    """|<a, b> - <c, d>| relative to the magnitude of the summands."""
    lhs, rhs = float(np.vdot(a, b)), float(np.vdot(c, d))
    scale = max(float(np.sum(np.abs(a * b))), float(np.sum(np.abs(c * d))), 1e-300)
    return abs(lhs - rhs) / scale


@pytest.mark.parametrize("name", ADJ_NAMES)
def test_vjp_dot_product(name, gpu_lib, pkg):
    host, u = cases.make(name)
    G = pkg.GB300Solver(host)
    T = O.TangentOracle(host)
    rng = np.random.default_rng(11)
    for _ in range(3):
        lam = rng.standard_normal(u.shape)
        v = rng.standard_normal(u.shape)
        mu = G.residual_vjp(u, lam)
        _, jv = T.jvp(u, v)
        assert _dot_rel(lam, jv, mu, v) < 1e-12


def test_vjp_full_transpose(gpu_lib, pkg):
    """Every entry of J^T lam against lam . (J e_i) from the tangent oracle."""
    pb = pkg.setups.vortex_tri(cells=8, p=2)
    host = pkg.solver.HostArrays(pb.law, pb.sd, pb.form)
    u = pkg.setups.perturbed(pb.u0, 7, 1e-3)
    G = pkg.GB300Solver(host)
    T = O.TangentOracle(host)
    lam = np.random.default_rng(12).standard_normal(u.shape)
    mu = G.residual_vjp(u, lam).ravel()
    want = np.empty(u.size)
    e = np.zeros(u.size)
    for i in range(u.size):
        e[i] = 1.0
        want[i] = float(np.vdot(lam.ravel(), T.jvp(u, e.reshape(u.shape))[1].ravel()))
        e[i] = 0.0
    scale = np.abs(want).max()
    assert np.abs(mu - want).max() < 1e-12 * scale


@pytest.mark.parametrize("name", ["adv_tri_modal", "adv_tri_nodal", "adv_tri_fd"])
def test_vjp_full_transpose_linear(name, gpu_lib, pkg):
    """Advection residuals are linear: J^T lam entry by entry against the
    tangent oracle's columns J e_i (StandardForm and FluxDifferencingForm)."""
    host, u = cases.make(name)
    G = pkg.GB300Solver(host)
    T = O.TangentOracle(host)
    lam = np.random.default_rng(13).standard_normal(u.shape)
    mu = G.residual_vjp(u, lam).ravel()
    want = np.empty(u.size)
    e = np.zeros(u.size)
    for i in range(u.size):
        e[i] = 1.0
        want[i] = float(np.vdot(lam.ravel(), T.jvp(u, e.reshape(u.shape))[1].ravel()))
        e[i] = 0.0
    assert np.abs(mu - want).max() < 1e-12 * np.abs(want).max()


def test_rk4_adjoint_standard_form(gpu_lib, pkg):
    """The advection workload's stepper (StandardForm, classic RK4) pulled
    back through checkpoints against the oracle trajectory's tangent."""
    pb = pkg.setups.advection_tri(cells=4, p=4)
    host = pkg.solver.HostArrays(pb.law, pb.sd, pb.form)
    u0 = pkg.setups.perturbed(pb.u0, 23, 1e-3)
    G = pkg.GB300Solver(host)
    uT = u0.copy()
    G.rk_record(uT, 6, pb.dt, 1, 4)
    rng = np.random.default_rng(24)
    lamT = rng.standard_normal(u0.shape)
    info = G.rk_adjoint(lamT)
    T = O.TangentOracle(host)
    v = rng.standard_normal(u0.shape)
    uT_o, w = T.rk_jvp(u0, v, 6, pb.dt, 1)
    assert _dot_rel(lamT, w, info["lam_0"], v) < 1e-11
    assert O.rel2(uT, uT_o) < 1e-12


def test_vjp_device_pointers_and_determinism(gpu_lib, pkg):
    import torch
    host, u = cases.make("tgv_tet_modal")
    G = pkg.GB300Solver(host)
    lam = np.random.default_rng(13).standard_normal(u.shape)
    ud = torch.from_numpy(u).cuda()
    ld = torch.from_numpy(lam).cuda()
    m1 = G.residual_vjp(ud, ld)
    m2 = G.residual_vjp(ud, ld)
    torch.cuda.synchronize()
    assert torch.equal(m1, m2)
    assert np.array_equal(m1.cpu().numpy(), G.residual_vjp(u, lam))


def _vortex(pkg, cells=8, p=3):
    pb = pkg.setups.vortex_tri(cells=cells, p=p)
    host = pkg.solver.HostArrays(pb.law, pb.sd, pb.form)
    return pb, host


@pytest.mark.parametrize("scheme,every", [(0, 3), (0, 0), (1, 2), (1, 7)])
def test_rk_adjoint_against_trajectory_tangent(scheme, every, gpu_lib, pkg):
    pb, host = _vortex(pkg)
    u0 = pkg.setups.perturbed(pb.u0, 21, 1e-3)
    n_steps = 7
    G = pkg.GB300Solver(host)
    uT = u0.copy()
    G.rk_record(uT, n_steps, pb.dt, scheme, every)
    rng = np.random.default_rng(22)
    lamT = rng.standard_normal(u0.shape)
    info = G.rk_adjoint(lamT)
    lam0 = info["lam_0"]
    assert info["segments"] * info["checkpoint_every"] >= n_steps
    T = O.TangentOracle(host)
    for _ in range(2):
        v = rng.standard_normal(u0.shape)
        uT_o, w = T.rk_jvp(u0, v, n_steps, pb.dt, scheme)
        assert _dot_rel(lamT, w, lam0, v) < 1e-11
    assert O.rel2(uT, uT_o) < 1e-12


def test_rk_adjoint_checkpoint_interval_invariance(gpu_lib, pkg):
    pb, host = _vortex(pkg)
    u0 = pkg.setups.perturbed(pb.u0, 23, 1e-3)
    G = pkg.GB300Solver(host)
    lamT = np.random.default_rng(24).standard_normal(u0.shape)
    grads = []
    for every in (1, 2, 5, 6, 0):
        u = u0.copy()
        G.rk_record(u, 6, pb.dt, 0, every)
        first = G.rk_adjoint(lamT)
        grads.append(first["lam_0"])
        nseg = first["segments"]
        # the recording run kept the last segment's stage data
        assert first["recomputed"] == nseg - 1
        # the recording stays valid for a second pullback, which recomputes
        # the last segment too when there are several
        second = G.rk_adjoint(lamT)
        assert second["recomputed"] == (nseg if nseg > 1 else 0)
        assert np.array_equal(second["lam_0"], grads[-1])
    for g in grads[1:]:
        assert np.array_equal(g, grads[0])


@pytest.mark.parametrize("scheme", [0, 1])
def test_binomial_schedule_matches_uniform_bitwise(scheme, gpu_lib, pkg):
    """sse_rk_record_binomial: the same gradient, bit for bit, as the uniform
    recording for any number of checkpoints; the final state is the forward
    run's; the first pullback recomputes the schedule's extra steps F(n, c),
    a second one (the descent's slots were reused) all n + F(n, c)."""
    pb, host = _vortex(pkg)
    u0 = pkg.setups.perturbed(pb.u0, 41, 1e-3)
    n_steps = 9
    G = pkg.GB300Solver(host)
    lamT = np.random.default_rng(42).standard_normal(u0.shape)
    uT = u0.copy()
    G.rk_record(uT, n_steps, pb.dt, scheme, 0)
    want = G.rk_adjoint(lamT)["lam_0"]
    for c in (0, 1, 2, 3, 8):
        u = u0.copy()
        G.rk_record_binomial(u, n_steps, pb.dt, scheme, c)
        assert np.array_equal(u, uT)
        first = G.rk_adjoint(lamT)
        extra, _ = pkg.gb300.binomial_schedule(n_steps, c if c else n_steps - 1)
        assert first["checkpoint_every"] == -1
        assert first["recomputed"] == extra, (c, first["recomputed"], extra)
        assert np.array_equal(first["lam_0"], want), c
        second = G.rk_adjoint(lamT)
        assert second["recomputed"] == n_steps + extra
        assert np.array_equal(second["lam_0"], want)
    # the uniform recording still works after a binomial one
    u = u0.copy()
    G.rk_record(u, n_steps, pb.dt, scheme, 4)
    assert np.array_equal(G.rk_adjoint(lamT)["lam_0"], want)


def test_binomial_schedule_against_trajectory_tangent(gpu_lib, pkg):
    pb, host = _vortex(pkg)
    u0 = pkg.setups.perturbed(pb.u0, 43, 1e-3)
    n_steps = 11
    G = pkg.GB300Solver(host)
    uT = u0.copy()
    G.rk_record_binomial(uT, n_steps, pb.dt, 0, 2)
    rng = np.random.default_rng(44)
    lamT = rng.standard_normal(u0.shape)
    lam0 = G.rk_adjoint(lamT)["lam_0"]
    T = O.TangentOracle(host)
    v = rng.standard_normal(u0.shape)
    uT_o, w = T.rk_jvp(u0, v, n_steps, pb.dt, 0)
    assert _dot_rel(lamT, w, lam0, v) < 1e-11
    assert O.rel2(uT, uT_o) < 1e-12


def test_binomial_schedule_mixed_recording(gpu_lib, pkg):
    """A mixed-form recording on the binomial schedule: the gradient of the
    uniform mixed recording, bit for bit, within 1e-4 of the FP64 one."""
    pb, host = _vortex(pkg)
    u0 = pkg.setups.perturbed(pb.u0, 45, 1e-3)
    G = pkg.GB300Solver(host)
    lamT = np.random.default_rng(46).standard_normal(u0.shape)
    u = u0.copy()
    G.rk_record(u, 6, pb.dt, 0, 2)
    g64 = G.rk_adjoint(lamT)["lam_0"]
    G.set_precision(pkg.abi.SSE_MIXED)
    u = u0.copy()
    G.rk_record(u, 6, pb.dt, 0, 0)
    gm = G.rk_adjoint(lamT)["lam_0"]
    ub = u0.copy()
    G.rk_record_binomial(ub, 6, pb.dt, 0, 2)
    gb = G.rk_adjoint(lamT)["lam_0"]
    assert np.array_equal(ub, u)
    assert np.array_equal(gb, gm)
    assert O.rel2(gb, g64) < 1e-4


@pytest.mark.parametrize("name", ["vortex_tri_modal", "tgv_tet_modal", "tgv_tet_ec", "tgv_tet_p5",
                                  "multi_tet", "tgv_tet_exact", "tgv_tet_ec_exact", "vortex_tri_exact"])
def test_mixed_vjp_against_fp64(name, gpu_lib, pkg):
    """The mixed-form VJP (FP32 transposes of the reduced fluxes and of the
    FP32 projection) against the FP64 VJP at the same state, and the
    dot-product identity against the dual-number oracle at FP32 accuracy,
    including meshes with exact metrics that do not preserve a free stream
    (the reference-pressure terms the FP32 fluxes leave out are constant in
    u, so the Jacobian is unchanged)."""
    host, u = cases.make(name)
    G = pkg.GB300Solver(host)
    rng = np.random.default_rng(31)
    lam = rng.standard_normal(u.shape)
    mu64 = G.residual_vjp(u, lam)
    G.set_precision(pkg.abi.SSE_MIXED)
    mu32 = G.residual_vjp(u, lam)
    err = O.rel2(mu32, mu64)
    assert err < 1e-4, err
    v = rng.standard_normal(u.shape)
    _, jv = O.TangentOracle(host).jvp(u, v)
    assert _dot_rel(lam, jv, mu32, v) < 1e-4


def test_rk_adjoint_mixed_recording(gpu_lib, pkg):
    pb, host = _vortex(pkg)
    u0 = pkg.setups.perturbed(pb.u0, 25, 1e-3)
    G = pkg.GB300Solver(host)
    lamT = np.random.default_rng(26).standard_normal(u0.shape)
    u = u0.copy()
    G.rk_record(u, 6, pb.dt, 0, 2)
    g64 = G.rk_adjoint(lamT)["lam_0"]
    G.set_precision(pkg.abi.SSE_MIXED)
    um = u0.copy()
    G.rk_record(um, 6, pb.dt, 0, 2)
    gm = G.rk_adjoint(lamT)["lam_0"]
    # the pullback of a mixed recording uses the mixed-form VJP
    assert O.rel2(um, u) < 1e-6
    assert O.rel2(gm, g64) < 1e-4


def test_gradient_against_central_differences(gpu_lib, pkg):
    """dJ/du0 for J = 1/2 ||u(T) - u_target||^2_M against central
    differences of J through the GPU forward along seeded directions."""
    pb, host = _vortex(pkg)
    tgt = pkg.setups.vortex_tri(cells=8, p=3, strength=5.5, shift=0.3)
    obj = pkg.objectives
    G = pkg.GB300Solver(host)
    u0 = pb.u0.copy()
    n_steps = 10

    def J(u):
        u = u.copy()
        G.rk_steps(u, n_steps, pb.dt, 0)
        return obj.mass_misfit(host, u, tgt.u0)

    uT = u0.copy()
    G.rk_record(uT, n_steps, pb.dt, 0, 4)
    _, dJdu = obj.mass_misfit(host, uT, tgt.u0)
    grad = G.rk_adjoint(dJdu)["lam_0"]
    rng = np.random.default_rng(27)
    for _ in range(4):
        v = rng.standard_normal(u0.shape)
        v /= np.linalg.norm(v)
        h = 1e-6
        fd = (J(u0 + h * v)[0] - J(u0 - h * v)[0]) / (2 * h)
        ad = float(np.vdot(grad, v))
        assert abs(fd - ad) <= 1e-5 * max(abs(ad), 1e-3 * np.linalg.norm(grad)), (fd, ad)


def test_c4_submesh_gradient_against_dual_numbers(gpu_lib, pkg):
    """The C4 adjoint configuration on its 4 x 4 sub-mesh (32 curved
    triangles, ModalTensor(4), FD + LF): J = 1/2 ||u(T) - u_target||^2_M
    after 400 CarpenterKennedy2N54 stages of C4's time step, checkpoints
    every 20 stages,
    u_target the perturbed vortex of strength 5.5 shifted by 0.3.  The GPU
    gradient against forward-mode dual numbers through the oracle's
    residual along 8 seeded directions: dJ . v = <M (u(T) - u_target),
    (du(T)/du(0)) v>."""
    pb = pkg.setups.vortex_tri(cells=4, p=4)
    host = pb.host_arrays()
    tgt = pkg.setups.perturbed(pkg.setups.vortex_tri(cells=4, p=4, strength=5.5, shift=0.3).u0,
                               20261207, 1e-3)
    obj = pkg.objectives
    # the time step of the C4 configuration itself (8192 triangles: h =
    # 10 / sqrt(N_p N_e), CFL 0.1 against |V| + c = sqrt(2) + 1)
    n_steps = 80
    dt = 0.1 * (10.0 / math.sqrt(15 * 8192)) / (math.sqrt(2.0) + 1.0)
    G = pkg.GB300Solver(host)
    uT = pb.u0.copy()
    G.rk_record(uT, n_steps, dt, 0, 4)
    _, dJ = obj.mass_misfit(host, uT, tgt)
    grad = G.rk_adjoint(dJ)["lam_0"]
    T = O.TangentOracle(host)
    rng = np.random.default_rng(20261208)
    for _ in range(8):
        v = rng.standard_normal(pb.u0.shape)
        uT_o, w = T.rk_jvp(pb.u0, v, n_steps, dt, 0)
        assert _dot_rel(dJ, w, grad, v) < 1e-11
    assert O.rel2(uT, uT_o) < 1e-12


def test_recording_larger_than_memory_is_refused(gpu_lib, pkg):
    """A recording that cannot fit is refused on the host before any step
    runs (the state is left as it was)."""
    host, u = cases.make("vortex_tri_modal")
    G = pkg.GB300Solver(host)
    u0 = u.copy()
    n = 2_000_000
    with pytest.raises(pkg.SSEError) as e:
        G.rk_record(u, n, 1e-6, 0, n)        # one segment of every stage: far above HBM
    assert e.value.code == pkg.abi.SSE_ERR_OUT_OF_MEMORY
    assert np.array_equal(u, u0)
    with pytest.raises(pkg.SSEError):
        G.rk_adjoint(u)                      # nothing recorded


def test_mixed_vjp_needs_a_modal_basis(gpu_lib, pkg):
    host, u = cases.make("vortex_tri_nodal")
    G = pkg.GB300Solver(host)
    G.set_precision(pkg.abi.SSE_MIXED)
    with pytest.raises(pkg.SSEError) as e:
        G.residual_vjp(u, u)
    assert e.value.code == pkg.abi.SSE_ERR_UNSUPPORTED


def test_adjoint_rejections(gpu_lib, pkg):
    """A pullback without a recording is refused, and so is the VJP of
    Chandrashekar's two-point flux (an extra forward option)."""
    host, u = cases.make("vortex_tri_modal")
    G = pkg.GB300Solver(host)
    with pytest.raises(pkg.SSEError) as e:
        G.rk_adjoint(u)
    assert e.value.code == pkg.abi.SSE_ERR_INVALID_ARGUMENT
    host, u = cases.make("vortex_tri_chandra")
    G = pkg.GB300Solver(host)
    with pytest.raises(pkg.SSEError) as e:
        G.residual_vjp(u, u)
    assert e.value.code == pkg.abi.SSE_ERR_UNSUPPORTED
