"""The reference's own end-to-end test scenarios on the hot path, set up
through the host mirror exactly as the reference's tests do.

advection_2d: test/runtests.jl:38-60 via test/test_driver.jl:1-110
  (ModalTensor(4) Tri, mapping_degree 4, 2x2 periodic cells on [0,1]^2,
  DelRey warp 0.1, ExactMetrics with project_jacobian, StandardForm with
  LaxFriedrichsNumericalFlux(0.0), CarpenterKennedy2N54 with dt = 0.01 to
  T = 1, solution saved every 2 steps).
euler_vortex_2d: test/euler_vortex_2d_modal.jl:1-73 (ModalTensor(3) Tri,
  4x4 cells, ChanWarping(1/16), ChanWilcoxMetrics, FluxDifferencingForm with
  Lax-Friedrichs, isentropic vortex, CarpenterKennedy2N54 with dt = T/1000).
"""
import math

import numpy as np

import __graft_entry__

PKG = __graft_entry__.load_package()
S, M, R = PKG.solver, PKG.mesh, PKG.reference


def l2_error(sd, u, exact):
    """ErrorAnalysis with the volume quadrature (Analysis/error.jl:58-91)."""
    return PKG.timestepping.l2_error(sd, u, lambda x, t: exact(x))


def advection_2d():
    ra = R.reference_approximation("ModalTensor", "Tri", 4, mapping_degree=4)
    mesh = M.uniform_periodic_mesh(ra, ((0.0, 1.0), (0.0, 1.0)), (2, 2))
    mesh = M.warp_mesh(mesh, ra, "DelRey", 0.1, (1.0, 1.0))
    sd = M.spatial_discretization(mesh, ra, "Exact", project_jac=True)
    law = S.LinearAdvectionEquation((1.0, 1.0))
    ic = S.InitialDataSine(1.0, (2 * math.pi, 2 * math.pi))
    form = S.StandardForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux(0.0))
    host = S.HostArrays(law, sd, form)
    u0 = S.initialize(ic, sd)
    exact = lambda x, T=1.0: ic.evaluate([x[0] - T, x[1] - T])
    return dict(host=host, sd=sd, u0=u0, dt=0.01, steps=100, save_every=2, exact=exact)


def euler_vortex_2d():
    Ma, L, gam = 0.4, 1.0, 1.4
    T = L / Ma
    strength = math.sqrt(2 / (gam - 1) * (1 - 0.75 ** (gam - 1)))
    ic = S.IsentropicVortex(gamma=gam, Ma=Ma, theta=0.0, R=0.1, beta=strength, sigma=1.0,
                            x0=(L / 2, L / 2))
    ra = R.reference_approximation("ModalTensor", "Tri", 3, mapping_degree=3)
    mesh = M.uniform_periodic_mesh(ra, ((0.0, L), (0.0, L)), (4, 4))
    mesh = M.warp_mesh(mesh, ra, "Chan", 1.0 / 16.0, (L, L))
    sd = M.spatial_discretization(mesh, ra, "ChanWilcox")
    law = S.EulerEquations(2, gam)
    form = S.FluxDifferencingForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
    host = S.HostArrays(law, sd, form)
    u0 = S.initialize(ic, sd)
    return dict(host=host, sd=sd, u0=u0, dt=T / 1000, steps=1000,
                save_every=int(math.floor(T / (T / 1000 * 50))), exact=lambda x: ic.evaluate(x))


def energy_rate_wa(host, u, du):
    """sum_k u' M dudt, M the weight-adjusted mass matrix (conservation.jl:161-175)."""
    V = host.sd.reference_approximation.V
    total = 0.0
    for k in range(host.N_e):
        Minv = V.T @ (host.JinvW[k][:, None] * V)
        total += u[k, 0] @ np.linalg.solve(Minv, du[k, 0])
    return total


def conserved_totals(host, u):
    """sum_k 1' WJ V u[:, e, k] (evaluate_conservation, conservation.jl:113-118)."""
    V = host.sd.reference_approximation.V_dense
    return np.einsum("kq,qp,kcp->c", host.WJ, V, u)
