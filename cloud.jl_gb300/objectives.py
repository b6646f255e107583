"""Objectives of the discrete-adjoint workloads and their gradients with
respect to the final state, evaluated on the host from the reference
approximation's dense Vandermonde and the quadrature weights W .* J.

These are caller-side functionals (what a user differentiates through the
stepper's pullback), evaluated on the host like the reference's Analysis
module (src/Analysis/conservation.jl:145-189 integrates states with the same
W .* J quadrature and V):

* ``mass_misfit``: J = 1/2 ||u - u_target||^2_M with M the element mass
  matrix V' diag(W J) V;
* ``kinetic_energy``: the volume-averaged kinetic energy
  (1/|Omega|) sum_k 1' (W J) (|m|^2 / (2 rho)) at the volume quadrature
  nodes of u_q = V u (the quadrature of 1/2 rho |V|^2; the reference has no
  such functional).
"""
from __future__ import annotations

import numpy as np

from .solver import HostArrays


def _V(host: HostArrays) -> np.ndarray:
    return host.sd.reference_approximation.V_dense


def mass_apply(host: HostArrays, x: np.ndarray) -> np.ndarray:
    """M x per element; x has the state layout (N_e, N_c, N_p)."""
    V = _V(host)
    xq = np.einsum("qp,ecp->ecq", V, x) * host.WJ[:, None, :]
    return np.einsum("qp,ecq->ecp", V, xq)


def mass_misfit(host: HostArrays, u: np.ndarray, u_target: np.ndarray):
    """(J, dJ/du) for J = 1/2 ||u - u_target||^2_M."""
    r = u - u_target
    Mr = mass_apply(host, r)
    return 0.5 * float(np.vdot(r, Mr)), Mr


def kinetic_energy(host: HostArrays, u: np.ndarray):
    """(KE, dKE/du) for the volume-averaged kinetic energy of an Euler state."""
    V = _V(host)
    uq = np.einsum("qp,ecp->ecq", V, u)
    rho, m = uq[:, 0], uq[:, 1:-1]
    m2 = np.sum(m * m, axis=1)
    vol = float(host.WJ.sum())
    ke = float(np.sum(host.WJ * 0.5 * m2 / rho)) / vol
    g = np.zeros_like(uq)
    g[:, 0] = -0.5 * m2 / rho ** 2
    g[:, 1:-1] = m / rho[:, None, :]
    g *= host.WJ[:, None, :] / vol
    return ke, np.einsum("qp,ecq->ecp", V, g)
