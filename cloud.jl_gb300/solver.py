"""Host mirror of the reference's solver-facing API.

Python counterparts of the Julia types the drop-in boundary sees:
conservation laws and numerical fluxes (src/ConservationLaws/
ConservationLaws.jl:51-73, euler_navierstokes.jl:26-38,
linear_advection_diffusion.jl:10-19), residual forms (src/Solvers/
Solvers.jl:90-115), initial data (src/GridFunctions/GridFunctions.jl,
euler_navierstokes.jl:234-320), ``initialize``/``project_function``
(Solvers.jl:388-427) and ``semidiscretize`` (Solvers.jl:429-452).

``build_host_arrays`` assembles exactly the fields of the reference's
``ReferenceOperators`` (operators.jl:1-37), ``FluxDifferencingOperators``
(operators.jl:39-81) and mass solvers (mass_matrix.jl:19-24, 59-115) as
contiguous FP64 arrays in the reference's column-major layouts; the GB300
library (``GB300Backend``) consumes them through the C-ABI.  The residual
itself never runs here: a ``Solver`` without its CUDA library raises.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import abi
from .mesh import SpatialDiscretization
from .reference import reference_derivative_operators


# ---------------------------------------------------------------------------
# conservation laws, fluxes, forms
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class LinearAdvectionEquation:
    a: tuple

    @property
    def d(self) -> int:
        return len(self.a)

    N_c = 1


@dataclass(frozen=True)
class EulerEquations:
    d: int
    gamma: float = 1.4

    @property
    def N_c(self) -> int:
        return self.d + 2


@dataclass(frozen=True)
class LaxFriedrichsNumericalFlux:
    lam: float = 1.0

    @property
    def half_lambda(self) -> float:
        return 0.5 * self.lam


@dataclass(frozen=True)
class CentralNumericalFlux:
    pass


@dataclass(frozen=True)
class EntropyConservativeNumericalFlux:
    pass


@dataclass(frozen=True)
class EntropyConservativeFlux:
    pass


@dataclass(frozen=True)
class ConservativeFlux:
    pass


@dataclass(frozen=True)
class ChandrashekarFlux:
    """Chandrashekar's (2013) entropy-conservative and kinetic-energy
    preserving two-point flux for the Euler equations: an extra option with
    no counterpart in the reference, whose entropy-conservative flux is
    Ranocha's (EntropyConservativeFlux)."""
    pass


@dataclass(frozen=True)
class StandardForm:
    inviscid_numerical_flux: object = field(default_factory=LaxFriedrichsNumericalFlux)


@dataclass(frozen=True)
class FluxDifferencingForm:
    inviscid_numerical_flux: object = field(default_factory=LaxFriedrichsNumericalFlux)
    two_point_flux: object = field(default_factory=EntropyConservativeFlux)


# ---------------------------------------------------------------------------
# initial data (GridFunctions.jl, euler_navierstokes.jl)
# ---------------------------------------------------------------------------

@dataclass(frozen=True)
class InitialDataSine:
    A: float
    k: tuple
    N_c = 1

    def evaluate(self, x, t=0.0):
        val = self.A * np.prod([np.sin(self.k[m] * x[m]) for m in range(len(self.k))], axis=0)
        return val[..., None]


@dataclass(frozen=True)
class IsentropicVortex:
    """euler_navierstokes.jl:234-266 (``evaluate`` ignores t there; the
    ``translated`` flag evaluates the exactly advected vortex instead)."""
    gamma: float = 1.4
    Ma: float = 0.4
    theta: float = math.pi / 4
    R: float = 1.0
    beta: float = 1.0
    sigma: float = 1.0
    x0: tuple = (0.0, 0.0)
    period: tuple | None = None
    N_c = 4

    def evaluate(self, x, t=0.0, translated=False):
        g = self.gamma
        xc = [self.x0[0], self.x0[1]]
        if translated:
            xc[0] += self.Ma * math.cos(self.theta) * t
            xc[1] += self.Ma * math.sin(self.theta) * t
        rel = []
        for m in range(2):
            dx = x[m] - xc[m]
            if translated and self.period is not None:
                L = self.period[m]
                dx = dx - L * np.rint(dx / L)
            rel.append(dx / self.R)
        omega = self.beta * np.exp(-0.5 / self.sigma ** 2 * (rel[0] ** 2 + rel[1] ** 2))
        dv = (-rel[1] * omega, rel[0] * omega)
        dT = -0.5 * (g - 1) * omega ** 2
        rho = (1 + dT) ** (1 / (g - 1))
        v = (self.Ma * math.cos(self.theta) + dv[0], self.Ma * math.sin(self.theta) + dv[1])
        p = rho ** g / g
        E = p / (g - 1) + 0.5 * rho * (v[0] ** 2 + v[1] ** 2)
        return np.stack([rho, rho * v[0], rho * v[1], E], axis=-1)


@dataclass(frozen=True)
class TaylorGreenVortex:
    """euler_navierstokes.jl:302-320."""
    gamma: float = 1.4
    Ma: float = 0.1
    N_c = 5

    def evaluate(self, x, t=0.0):
        g = self.gamma
        p = (1 / (self.Ma ** 2 * g)) + 0.0625 * (
            2 * np.cos(2 * x[0]) + 2 * np.cos(2 * x[1]) + np.cos(2 * x[0]) * np.cos(2 * x[2])
            + np.cos(2 * x[1]) * np.cos(2 * x[2]))
        u = np.sin(x[0]) * np.cos(x[1]) * np.cos(x[2])
        v = -np.cos(x[0]) * np.sin(x[1]) * np.cos(x[2])
        one = np.ones_like(u)
        return np.stack([one, u, v, np.zeros_like(u), p / (g - 1) + 0.5 * (u ** 2 + v ** 2)], axis=-1)


@dataclass(frozen=True)
class EulerPeriodicTest:
    """euler_navierstokes.jl:276-294."""
    d: int
    gamma: float = 1.4
    strength: float = 0.2
    L: float = 2.0

    @property
    def N_c(self):
        return self.d + 2

    def evaluate(self, x, t=0.0):
        rho = 1.0 + self.strength * np.sin(2 * np.pi * sum(x[m] for m in range(self.d)) / self.L)
        cols = [rho] + [rho] * self.d + [1.0 / (self.gamma - 1.0) + 0.5 * rho * self.d]
        return np.stack([np.broadcast_to(c, rho.shape) for c in cols], axis=-1)


# ---------------------------------------------------------------------------
# initialize (Solvers.jl:388-427)
# ---------------------------------------------------------------------------

def initialize(initial_data, sd: SpatialDiscretization, projection: str = "host") -> np.ndarray:
    """L2 projection of the initial data onto the approximation space;
    returns numpy (N_e, N_c, N_p) = Julia (N_p, N_c, N_e).
    ``projection="gpu"`` solves the element mass systems on the GPU
    (sse_project_function) instead of numpy."""
    ra = sd.reference_approximation
    x = sd.mesh.xyzq
    uq = initial_data.evaluate(x, 0.0)                  # (N_e, N_q, N_c)
    if ra.V is None:
        return np.ascontiguousarray(uq.transpose(0, 2, 1))
    if projection == "gpu":
        from . import gb300
        return gb300.project_function(ra, sd.geometric_factors.J_q,
                                      np.ascontiguousarray(uq.transpose(0, 2, 1)))
    if projection != "host":
        raise ValueError(projection)
    V = ra.V
    WJ = ra.W[None, :] * sd.geometric_factors.J_q       # (N_e, N_q)
    out = np.empty((sd.N_e, uq.shape[2], ra.N_p))
    Np = ra.N_p
    # M_k[a, b] = sum_q WJ[k, q] V[q, a] V[q, b]: one GEMM against the
    # products of Vandermonde columns
    VV = (V[:, :, None] * V[:, None, :]).reshape(V.shape[0], Np * Np)
    chunk = 8192
    for s in range(0, sd.N_e, chunk):
        e = min(sd.N_e, s + chunk)
        M = (WJ[s:e] @ VV).reshape(e - s, Np, Np)
        rhs = np.stack([(WJ[s:e] * uq[s:e, :, c]) @ V for c in range(uq.shape[2])], axis=-1)
        out[s:e] = np.linalg.solve(M, rhs).transpose(0, 2, 1)
    return out


# ---------------------------------------------------------------------------
# operator / geometry arrays handed across the C-ABI
# ---------------------------------------------------------------------------

class HostArrays:
    """Contiguous host copies of the reference's operator structs plus the
    ctypes structs pointing at them (kept alive together)."""

    def __init__(self, law, sd: SpatialDiscretization, form, mass_matrix_solver="default"):
        ra = sd.reference_approximation
        gf = sd.geometric_factors
        d = ra.d
        N_e = sd.N_e
        self.law = law
        self.form = form
        self.sd = sd
        fd = isinstance(form, FluxDifferencingForm)
        nflux = form.inviscid_numerical_flux
        if isinstance(nflux, LaxFriedrichsNumericalFlux):
            nf_kind, half_lambda = abi.SSE_LAX_FRIEDRICHS, nflux.half_lambda
        elif isinstance(nflux, CentralNumericalFlux):
            nf_kind, half_lambda = abi.SSE_CENTRAL, 0.0
        elif isinstance(nflux, EntropyConservativeNumericalFlux):
            nf_kind, half_lambda = abi.SSE_ENTROPY_CONSERVATIVE, 0.0
        else:
            raise ValueError(f"unsupported numerical flux {nflux}")
        two_pt = abi.SSE_EC_FLUX
        if fd and isinstance(form.two_point_flux, ConservativeFlux):
            two_pt = abi.SSE_CONSERVATIVE_FLUX
        if fd and isinstance(form.two_point_flux, ChandrashekarFlux):
            two_pt = abi.SSE_CHANDRASHEKAR_FLUX
        mass = abi.SSE_DIAGONAL if ra.V is None else abi.SSE_WEIGHT_ADJUSTED
        if mass_matrix_solver not in ("default", "WeightAdjusted", "Diagonal"):
            raise ValueError(mass_matrix_solver)
        if isinstance(law, EulerEquations):
            law_kind, gamma, a = abi.SSE_EULER, law.gamma, (0.0, 0.0, 0.0)
        else:
            law_kind, gamma = abi.SSE_LINEAR_ADVECTION, 0.0
            a = tuple(law.a) + (0.0,) * (3 - len(law.a))
        self.N_p, self.N_q, self.N_f, self.N_c, self.N_e = ra.N_p, ra.N_q, ra.N_f, law.N_c, N_e
        self.cfg = abi.SseConfig(
            d=d, n_p=ra.N_p, n_q=ra.N_q, n_f=ra.N_f, n_c=law.N_c, n_e=N_e,
            num_faces=ra.reference_element.num_faces, nodes_per_face=ra.nodes_per_face,
            form=abi.SSE_FLUX_DIFFERENCING_FORM if fd else abi.SSE_STANDARD_FORM,
            law=law_kind, numerical_flux=nf_kind, two_point_flux=two_pt, mass_solver=mass,
            reserved=0, half_lambda=half_lambda, gamma=gamma, a=(abi.C.c_double * 3)(*a))

        # ---- reference operators
        ops = abi.SseOperators()
        if ra.warped is not None:
            wp = ra.warped
            self.vdm_A = np.ascontiguousarray(wp.A.T)          # Julia M1 x (p+1)
            self.vdm_B = np.ascontiguousarray(wp.B.transpose(2, 1, 0))
            self.vdm_C = (np.ascontiguousarray(wp.C.transpose(3, 2, 1, 0))
                          if wp.C is not None else None)
            self.vdm_sigma = np.ascontiguousarray((wp.sigma_in + 1).T)
            ops.vdm_p = wp.p
            for m, n in enumerate(ra.n1d):
                ops.vdm_m[m] = n
            ops.vdm_A = abi.dptr(self.vdm_A)
            ops.vdm_B = abi.dptr(self.vdm_B)
            ops.vdm_C = abi.dptr(self.vdm_C)
            ops.vdm_sigma_in = abi.iptr(self.vdm_sigma)
        elif ra.V is not None:
            # ModalMulti: Matrix(V), N_q x N_p column-major
            self.V_dense = np.ascontiguousarray(ra.V.T)
            ops.vdm_p = ra.p
            ops.V_dense = abi.dptr(self.V_dense)
        self.R = abi.CscArrays(ra.R)
        ops.R = self.R.struct()
        self.D = [abi.CscArrays(Dm) for Dm in ra.D]
        self.S = []
        self.C = None
        for m in range(3):
            ops.D[m] = self.D[m].struct() if (m < d and not fd) else abi.empty_csc()
        if fd:
            Dxi = reference_derivative_operators(ra)
            W = np.diag(ra.W)
            self.S = [abi.CscArrays(0.5 * (W @ Dxi[m] - Dxi[m].T @ W)) for m in range(d)]
            self.C = abi.CscArrays(ra.R.T @ np.diag(ra.B))
            for m in range(3):
                ops.S[m] = self.S[m].struct() if m < d else abi.empty_csc()
            ops.C = self.C.struct()
        else:
            for m in range(3):
                ops.S[m] = abi.empty_csc()
            ops.C = abi.empty_csc()
        self.ops = ops

        # ---- geometry (numpy shapes are the Julia shapes reversed)
        J_q = gf.J_q
        self.WJ = np.ascontiguousarray(ra.W[None, :] * J_q)
        self.BJf = np.ascontiguousarray(ra.B[None, :] * gf.J_f)
        self.n_f = np.ascontiguousarray(gf.nJf / gf.J_f[:, :, None])
        self.mapP = np.ascontiguousarray(sd.mesh.mapP.astype(np.int64))
        self.JinvW = np.ascontiguousarray(ra.W[None, :] / J_q) if mass == abi.SSE_WEIGHT_ADJUSTED else None
        self.WJinv = np.ascontiguousarray(1.0 / (ra.W[None, :] * J_q)) if mass == abi.SSE_DIAGONAL else None
        self.halfWLambda = None
        self.Lambda_q = None
        self.halfnJf = None
        self.halfnJq = None
        if fd:
            self.Lambda_q = np.ascontiguousarray(gf.Lambda_q)
            self.halfnJf = np.ascontiguousarray(0.5 * gf.nJf)
            self.halfnJq = np.ascontiguousarray(0.5 * gf.nJq)
        else:
            # apply_reference_mapping (SpatialDiscretizations.jl:398-411):
            # L_eta[i,m,n,k] = sum_l Lambda_ref[i,m,l] Lambda_q[i,l,n,k] / J_ref[i]
            Lref = ra.Lambda_ref                       # (N_q, m, l)
            Lq = gf.Lambda_q                           # [k, n, l, i]
            Leta = np.zeros_like(Lq)                   # [k, n, m, i]
            for m in range(d):
                acc = None
                for l in range(d):
                    term = Lref[:, m, l][None, None, :] * Lq[:, :, l, :] / ra.J_ref[None, None, :]
                    acc = term if acc is None else acc + term
                Leta[:, :, m, :] = acc
            self.Lambda_eta = Leta
            self.halfWLambda = np.ascontiguousarray(0.5 * ra.W[None, None, None, :] * Leta)
        geo = abi.SseGeometry()
        geo.BJf = abi.dptr(self.BJf)
        geo.n_f = abi.dptr(self.n_f)
        geo.mapP = abi.iptr(self.mapP)
        geo.halfWLambda = abi.dptr(self.halfWLambda)
        geo.WJ = abi.dptr(self.WJ)
        geo.Lambda_q = abi.dptr(self.Lambda_q)
        geo.halfnJf = abi.dptr(self.halfnJf)
        geo.halfnJq = abi.dptr(self.halfnJq)
        geo.JinvW = abi.dptr(self.JinvW)
        geo.WJinv = abi.dptr(self.WJinv)
        self.geo = geo

    @property
    def state_shape(self):
        """numpy shape of u / dudt: Julia (N_p, N_c, N_e) reversed."""
        return (self.N_e, self.N_c, self.N_p)

    @property
    def dof(self) -> int:
        """get_dof product N_p * N_c * N_e (Solvers.jl:381-386)."""
        return self.N_p * self.N_c * self.N_e
