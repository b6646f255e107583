"""Host-driven fixed-step time integration around the drop-in residual, and
the L2 error analysis of a solution.

``solve`` is what OrdinaryDiffEq does with the ODEProblem that
``semidiscretize`` returns (src/Solvers/Solvers.jl:429-452): for
``solve(ode, CarpenterKennedy2N54(); dt, adaptive=false)`` or ``RK4()`` it
calls the right-hand side ``semi_discrete_residual!(dudt, u, solver, t)``
once per stage on the integrator's own (host) arrays and does the stage
arithmetic on the host.  With the GB300 drop-in every stage therefore copies
u to the device and dudt back (``sse_residual`` with host pointers).  The
fused device loop ``GB300Solver.rk_steps`` (``sse_rk_steps``) is the faster
alternative that keeps the state resident; this driver measures what a
user of the unchanged Julia API gets.

The stage arithmetic runs in place: on torch CPU tensors (pinned memory, so
the library's copies are direct) with torch's intra-op threads, standing in
for OrdinaryDiffEq's broadcasts, or on numpy arrays.

``l2_error`` restates ``analyze(::ErrorAnalysis, sol, exact_solution, t)``
with the default (volume) quadrature (src/Analysis/error.jl:15-91).
"""
from __future__ import annotations

import numpy as np

# Carpenter & Kennedy (1994), NASA TM-109112: five-stage fourth-order
# 2N-storage coefficients (OrdinaryDiffEq's CarpenterKennedy2N54).
CK_A = (0.0, -567301805773.0 / 1357537059087.0, -2404267990393.0 / 2016746695238.0,
        -3550918686646.0 / 2091501179385.0, -1275806237668.0 / 842570457699.0)
CK_B = (1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
        1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
        2277821191437.0 / 14882151754819.0)


def _stage_times():
    """Stage abscissae of the 2N scheme: the recurrence applied to dy/dt = 1
    advances y exactly with time, so y before stage i is c_i."""
    c, y, q = [], 0.0, 0.0
    for a, b in zip(CK_A, CK_B):
        c.append(y)
        q = a * q + 1.0
        y += b * q
    return tuple(c)


CK_C = _stage_times()


class _Ops:
    """In-place axpy-type updates on numpy arrays or torch CPU tensors."""

    def __init__(self, u):
        self.torch = not isinstance(u, np.ndarray)
        if self.torch and u.is_cuda:
            raise ValueError("solve drives the residual from host arrays; use rk_steps for device state")

    def empty(self, u):
        if self.torch:
            return u.new_empty(u.shape).pin_memory() if u.is_pinned() else u.new_empty(u.shape)
        return np.empty_like(u)

    def axpy_into(self, q, a, k):
        """q <- a q + k (one pass on torch tensors)"""
        if self.torch:
            import torch
            torch.add(k, q, alpha=a, out=q)
        else:
            q *= a
            q += k

    def add_scaled(self, u, q, c, scratch):
        """u <- u + c q (one pass on torch tensors)"""
        if self.torch:
            u.add_(q, alpha=c)
        else:
            np.multiply(q, c, out=scratch)
            u += scratch

    def lincomb(self, y, x, b, z):
        """y <- x + b z (one pass on torch tensors)"""
        if self.torch:
            import torch
            torch.add(x, z, alpha=b, out=y)
        else:
            np.multiply(z, b, out=y)
            y += x


def solve(ode, dt: float, n_steps: int, alg: str = "CarpenterKennedy2N54", u=None, t0: float | None = None):
    """Advance ``u`` (default: a copy of ``ode.u0``) by ``n_steps`` fixed
    steps of ``alg`` ("CarpenterKennedy2N54" or "RK4"), calling
    ``ode.f(dudt, u, ode.p, t)`` once per stage.  Returns (u, t)."""
    if u is None:
        u = ode.u0.copy() if isinstance(ode.u0, np.ndarray) else ode.u0.clone()
    t = ode.tspan[0] if t0 is None else t0
    ops = _Ops(u)
    k = ops.empty(u)
    scratch = ops.empty(u)
    if alg == "CarpenterKennedy2N54":
        # the 2N recurrence q <- a q + dt k, u <- u + b q on the register
        # scaled by 1/dt (q' <- a q' + k, u <- u + (b dt) q'): two passes
        # over the state per stage, as OrdinaryDiffEq's fused broadcasts; on
        # the first stage (a = 0) the residual buffer itself becomes q'
        q = ops.empty(u)
        for _ in range(n_steps):
            for s, (a, b, c) in enumerate(zip(CK_A, CK_B, CK_C)):
                ode.f(k, u, ode.p, t + c * dt)
                if s == 0:
                    q, k = k, q
                else:
                    ops.axpy_into(q, a, k)
                ops.add_scaled(u, q, b * dt, scratch)
            t += dt
    elif alg == "RK4":
        # one fused pass per update: the stage states ust = u + c k, the
        # accumulator acc = k1 + 2 k2 + 2 k3 + k4 (k1's buffer becomes acc),
        # and u <- u + dt/6 (acc + k4)
        acc, ust = ops.empty(u), ops.empty(u)
        for _ in range(n_steps):
            ode.f(k, u, ode.p, t)
            acc, k = k, acc
            ops.lincomb(ust, u, 0.5 * dt, acc)
            ode.f(k, ust, ode.p, t + 0.5 * dt)
            ops.add_scaled(acc, k, 2.0, scratch)
            ops.lincomb(ust, u, 0.5 * dt, k)
            ode.f(k, ust, ode.p, t + 0.5 * dt)
            ops.add_scaled(acc, k, 2.0, scratch)
            ops.lincomb(ust, u, dt, k)
            ode.f(k, ust, ode.p, t + dt)
            ops.add_scaled(acc, k, 1.0, scratch)
            ops.add_scaled(u, acc, dt / 6.0, scratch)
            t += dt
    else:
        raise ValueError(f"unknown time integrator {alg!r}")
    return u, t


def l2_error(sd, u, exact, t: float = 0.0, normalize: bool = False) -> np.ndarray:
    """Quadrature L2 error of every conserved variable of ``u`` (numpy
    (N_e, N_c, N_p)) against ``exact(xyzq, t)`` (returning (N_e, N_q, N_c)),
    with the volume quadrature W and J_q; ``normalize`` divides by the
    domain volume before the square root (error.jl:58-91)."""
    ra = sd.reference_approximation
    ue = exact(sd.mesh.xyzq, t)
    ua = np.einsum("qp,kcp->kqc", ra.V_dense, u)
    w = ra.W[None, :, None] * sd.geometric_factors.J_q[:, :, None]
    err = ((ue - ua) ** 2 * w).sum(axis=(0, 1))
    if normalize:
        err = err / float((ra.W[None, :] * sd.geometric_factors.J_q).sum())
    return np.sqrt(err)
