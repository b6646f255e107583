"""The host-driven time integrator (``solve``: one right-hand-side call per
stage on host arrays, as OrdinaryDiffEq drives ``semi_discrete_residual!``)
and the L2 error analysis, without a GPU: fourth-order convergence of both
schemes on a linear ODE, the stage abscissae of the 2N scheme, agreement
with the oracle's own time stepping when the oracle is the right-hand side,
and numpy / torch-CPU agreement."""
import math

import numpy as np
import pytest

import cases
from oracle.oracle import Oracle, rel2

TS = cases.PKG.timestepping


class _Ode:
    def __init__(self, f, u0):
        self.f, self.u0, self.tspan, self.p = f, u0, (0.0, 1.0), None


def _linear(lam):
    def f(dudt, u, p, t):
        dudt[...] = lam * u
    return f


@pytest.mark.parametrize("alg", ["CarpenterKennedy2N54", "RK4"])
def test_fourth_order_on_a_linear_ode(alg):
    lam = np.array([-1.0, -0.3, 0.7])
    u0 = np.ones(3)
    errs = []
    for n in (10, 20, 40):
        u, t = TS.solve(_Ode(_linear(lam), u0), 1.0 / n, n, alg)
        assert abs(t - 1.0) < 1e-14
        errs.append(np.abs(u - np.exp(lam)).max())
    rates = [math.log2(errs[i] / errs[i + 1]) for i in range(2)]
    assert min(rates) > 3.8, rates


def test_stage_times_integrate_time_exactly():
    seen = []

    def f(dudt, u, p, t):
        seen.append(t)
        dudt[...] = 1.0
    u, t = TS.solve(_Ode(f, np.zeros(1)), 0.5, 1)
    assert abs(u[0] - 0.5) < 1e-15
    assert np.allclose(np.array(seen) / 0.5, TS.CK_C, atol=1e-15)
    assert TS.CK_C[0] == 0.0 and abs(TS.CK_C[1] - TS.CK_B[0]) < 1e-16


@pytest.mark.parametrize("name,scheme", [("vortex_tri_modal", 0), ("adv_tri_modal", 1)])
def test_host_driver_matches_oracle_stepping(name, scheme):
    host, u = cases.make(name)
    o = Oracle(host)

    def f(dudt, x, p, t):
        dudt[...] = o.residual(x)
    dt = 1e-3
    got, _ = TS.solve(_Ode(f, u), dt, 3, "RK4" if scheme else "CarpenterKennedy2N54")
    want = o.rk_steps(u.copy(), 3, dt, scheme)
    assert rel2(got, want) <= 1e-13


def test_numpy_and_torch_cpu_agree():
    torch = pytest.importorskip("torch")
    lam = np.linspace(-2.0, 1.0, 64)
    u0 = np.cos(lam)

    def f(dudt, u, p, t):
        dudt[...] = u * torch.from_numpy(lam) if not isinstance(u, np.ndarray) else u * lam
    for alg in ("CarpenterKennedy2N54", "RK4"):
        a, _ = TS.solve(_Ode(f, u0), 0.1, 5, alg)
        b, _ = TS.solve(_Ode(f, torch.from_numpy(u0.copy())), 0.1, 5, alg)
        assert np.abs(a - b.numpy()).max() <= 1e-14


def test_l2_error_of_the_projected_exact_solution_is_small():
    pb = cases.setups.vortex_tri(cells=8, p=4)
    ic = pb.initial_data
    err = TS.l2_error(pb.sd, pb.u0, lambda x, t: ic.evaluate(x, t))
    err_t = TS.l2_error(pb.sd, pb.u0, lambda x, t: ic.evaluate(x, t, translated=True))
    assert np.all(err < 0.1) and np.allclose(err, err_t)
    # the projection error converges at high order under refinement
    fine = cases.setups.vortex_tri(cells=16, p=4)
    err_f = TS.l2_error(fine.sd, fine.u0, lambda x, t: ic.evaluate(x, t))
    assert np.all(err_f < err / 8.0)
    # normalised by the domain volume (100)
    errn = TS.l2_error(pb.sd, pb.u0, lambda x, t: ic.evaluate(x, t), normalize=True)
    assert np.allclose(errn, err / 10.0)
