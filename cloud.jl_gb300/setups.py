"""Named workloads: the reference's test scenarios and the benchmark
configurations, assembled through the host mirror exactly as a reference
user would (ReferenceApproximation -> uniform_periodic_mesh -> warp_mesh ->
SpatialDiscretization -> semidiscretize).

Sizes:
  advection_tri   2-D linear advection, velocity (1,1), 16x16 periodic cells
                  -> 512 curved triangles, ModalTensor(4), StandardForm + LF,
                  sin(2 pi x) sin(2 pi y) on [0,1]^2, RK4 at CFL 0.1.
  vortex_tri      2-D Euler isentropic vortex on [0,10]^2, 64x64 cells ->
                  8192 curved triangles (Chan warp 0.1), ModalTensor(4),
                  FluxDifferencingForm (entropy-conservative volume flux + LF).
  tgv_tet         3-D Euler Taylor-Green vortex (Mach 0.1) on [0,2 pi]^3,
                  16^3 cells x 6 = 24,576 curved tets (Chan warp 0.05),
                  ModalTensor(4), FluxDifferencingForm, EC flux + LF or EC only.
  tgv_tet_p5      24^3 x 6 = 82,944 tets, ModalTensor(5), FD + LF.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from . import mesh as M
from . import reference as R
from . import solver as S


@dataclass
class Problem:
    name: str
    law: object
    sd: M.SpatialDiscretization
    form: object
    initial_data: object
    u0: np.ndarray
    dt: float
    scheme: int            # 0 = CarpenterKennedy2N54, 1 = RK4
    stages_per_step: int

    def host_arrays(self) -> S.HostArrays:
        return S.HostArrays(self.law, self.sd, self.form)


def multi_rules(shape: str, p: int):
    """Collapsed Gauss rules for ModalMulti / NodalMulti (the tabulated
    default rules are not restated): Tri LG(p) x LG(p) with LG(p) edges; Tet
    LG(p) x LG(p) x GJ(1,0)(p) with LG(p) x GJ(1,0)(p) faces."""
    if shape == "Tri":
        return (R.LGQuadrature(p), R.LGQuadrature(p)), R.LGQuadrature(p)
    return ((R.LGQuadrature(p), R.LGQuadrature(p), R.GaussRule(p, 1, 0)),
            (R.LGQuadrature(p), R.GaussRule(p, 1, 0)))


def _disc(approx, shape, p, limits, cells, warp_kind, warp_factor, metrics):
    if approx in ("ModalMulti", "NodalMulti"):
        vol, fac = multi_rules(shape, p)
        ra = R.reference_approximation(approx, shape, p, mapping_degree=p,
                                       volume_quadrature_rule=vol, facet_quadrature_rule=fac)
    else:
        ra = R.reference_approximation(approx, shape, p, mapping_degree=p)
    mesh = M.uniform_periodic_mesh(ra, limits, cells)
    L = tuple(hi - lo for lo, hi in limits)
    if warp_factor:
        mesh = M.warp_mesh(mesh, ra, warp_kind, warp_factor, L)
    return M.spatial_discretization(mesh, ra, metrics=metrics)


def advection_tri(cells: int = 16, p: int = 4, approx: str = "ModalTensor") -> Problem:
    sd = _disc(approx, "Tri", p, ((0.0, 1.0), (0.0, 1.0)), (cells, cells), "Chan", 0.1, "Exact")
    law = S.LinearAdvectionEquation((1.0, 1.0))
    ic = S.InitialDataSine(1.0, (2 * math.pi, 2 * math.pi))
    form = S.StandardForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
    u0 = S.initialize(ic, sd)
    ra = sd.reference_approximation
    h = 1.0 / math.sqrt(ra.N_p * sd.N_e)
    dt = 0.1 * h / math.sqrt(2.0)
    return Problem("advection_tri", law, sd, form, ic, u0, dt, 1, 4)


def vortex_tri(cells: int = 64, p: int = 4, approx: str = "ModalTensor",
               strength: float = 5.0, shift: float = 0.0, metrics: str = "ChanWilcox") -> Problem:
    """Isentropic vortex of strength 5 in a (1,1) free stream: the
    reference's ``IsentropicVortex`` with Ma = sqrt(2), theta = pi/4, R = 1,
    sigma = 1, beta = strength * e^{1/2} / (2 pi) (the classical Gaussian
    vortex velocity eps/(2 pi) exp((1-r^2)/2)), centred in [0,10]^2.
    ``metrics`` "ChanWilcox" (conservative curl) or "Exact", the
    reference's default."""
    L = 10.0
    sd = _disc(approx, "Tri", p, ((0.0, L), (0.0, L)), (cells, cells), "Chan", 0.1, metrics)
    law = S.EulerEquations(2, 1.4)
    ic = S.IsentropicVortex(gamma=1.4, Ma=math.sqrt(2.0), theta=math.pi / 4, R=1.0,
                            beta=strength * math.exp(0.5) / (2 * math.pi), sigma=1.0,
                            x0=(0.5 * L + shift, 0.5 * L + shift), period=(L, L))
    form = S.FluxDifferencingForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
    u0 = S.initialize(ic, sd)
    ra = sd.reference_approximation
    h = L / math.sqrt(ra.N_p * sd.N_e)
    dt = 0.1 * h / (math.sqrt(2.0) + 1.0)
    return Problem("vortex_tri", law, sd, form, ic, u0, dt, 0, 5)


def tgv_tet(cells: int = 16, p: int = 4, approx: str = "ModalTensor", lf: bool = True,
            metrics: str = "ChanWilcox") -> Problem:
    """``metrics`` "ChanWilcox" (conservative curl: a constant state is
    preserved to round-off, needed for round-off entropy conservation) or
    "Exact", the reference's default, which on these curved tets does not
    preserve a free stream."""
    L = 2 * math.pi
    sd = _disc(approx, "Tet", p, ((0.0, L),) * 3, (cells,) * 3, "Chan", 0.05, metrics)
    law = S.EulerEquations(3, 1.4)
    ic = S.TaylorGreenVortex(1.4, 0.1)
    nflux = S.LaxFriedrichsNumericalFlux() if lf else S.EntropyConservativeNumericalFlux()
    form = S.FluxDifferencingForm(inviscid_numerical_flux=nflux)
    u0 = S.initialize(ic, sd)
    ra = sd.reference_approximation
    h = L / (ra.N_p * sd.N_e) ** (1.0 / 3.0)
    c_max = math.sqrt(1.4 * (1 / (0.1 ** 2 * 1.4) + 0.25)) + 1.0
    dt = 0.1 * h / c_max
    return Problem("tgv_tet", law, sd, form, ic, u0, dt, 0, 5)


def perturbed(u0: np.ndarray, seed: int, scale: float = 1.0e-3) -> np.ndarray:
    """Parity input: the configuration's initial state plus a seeded
    perturbation scale*N(0,1) of every modal coefficient."""
    rng = np.random.default_rng(seed)
    return u0 + scale * rng.standard_normal(u0.shape)
