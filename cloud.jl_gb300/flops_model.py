"""Algorithmic work model of one residual evaluation, per element.

Counting convention: add, subtract, multiply = 1 flop; fused multiply-add =
2; divide, square root, log, exp, pow = 1 each.  Volume fluxes are counted
once per unique node pair, contractions once per (pair, direction)
incidence, as the reference's sparse loops perform them
(flux_differencing_form.jl:37-75, 126-168).  Bytes are the minimal HBM
traffic of the FP64 form: every array read or written once per phase,
the per-element dense mass operator included where a phase applies it.
The same numbers feed ``roofline.achieved`` in bench.py and the reports.
"""
from __future__ import annotations

from dataclasses import dataclass


@dataclass
class Work:
    flops_A: float      # nodal values / entropy projection, per element
    flops_B: float      # time derivative, per element
    bytes_A: float
    bytes_B: float
    bytes_stage: float  # Runge-Kutta stage update, per element

    @property
    def flops(self):
        return self.flops_A + self.flops_B

    @property
    def bytes(self):
        return self.bytes_A + self.bytes_B + self.bytes_stage


def vdm_flops(ra) -> float:
    """One sum-factorised application of V (or V^T) to one component."""
    if ra.V is None:
        return 0.0
    if ra.warped is None:
        return 2.0 * ra.N_q * ra.N_p          # dense V (ModalMulti)
    p1 = ra.p + 1
    if ra.d == 2:
        M1, M2 = ra.n1d
        return 2.0 * (M2 * ra.N_p + M1 * M2 * p1)
    M1, M2, M3 = ra.n1d
    nb12 = p1 * (p1 + 1) // 2
    return 2.0 * (M3 * ra.N_p + nb12 * M2 * M3 + M1 * p1 * M2 * M3)


def mass_solve_flops(ra) -> float:
    """One weight-adjusted mass solve of one component.  The reference
    applies V and V^T around the weighted diagonal (mass_matrix.jl:185-196);
    the kernels apply the precomputed per-element operator V^T diag(W/J) V,
    a dense n_p x n_p product.  The cheaper of the two is counted, so the
    model never credits work that is not done."""
    if ra.V is None:
        return 0.0
    return min(2.0 * vdm_flops(ra), 2.0 * ra.N_p * ra.N_p)


def ec_flux_flops(d: int) -> float:
    """Ranocha's two-point flux tensor from per-node primitives
    (euler_navierstokes.jl:171-195; logmean series branch)."""
    logmeans = 2 * 19
    return logmeans + 2 * d + (2 * d - 1) + 2 + 4 + d + 3 * d * d + 6 * d


def model(host) -> Work:
    """Work per element for the configuration held by ``host`` (HostArrays)."""
    ra = host.sd.reference_approximation
    d, nc, nq, nf, np_ = ra.d, host.N_c, host.N_q, host.N_f, host.N_p
    nnzR = host.R.nnz
    vf = vdm_flops(ra)
    mf = mass_solve_flops(ra)
    mb = 8.0 * np_ * np_ if ra.V is not None else 0.0   # the element's dense mass operator
    euler = nc > 1
    fd = host.S != []
    f8 = 8.0
    # ---- phase A
    if fd and euler:
        c2e = 3 * d + 12
        e2c = nc + 3 * d + 14
        nV = 3 if ra.V is not None else 0                # V u, V^T, V (+ one mass solve)
        flops_A = nc * (nV * vf + mf) + nc * 2 * nnzR + nq * (c2e + nc) + nq * nc + (nq + nf) * e2c
        bytes_A = f8 * (np_ * nc + 2 * nq + nq * nc + nf * nc) + mb
    else:
        flops_A = nc * (vf + 2 * nnzR)
        bytes_A = f8 * (np_ * nc + nq * nc + nf * nc)
    # ---- phase B
    nV_B = 1 if ra.V is not None else 0                  # V^T (+ one mass solve)
    if fd:
        S_inc = sum(s.nnz for s in host.S) // 2          # (pair, m) incidences with i < j
        pairs = _unique_pairs(host)
        nfp = host.C.nnz if host.C is not None else 0
        if euler:
            prim = 3 * d + 4
            pair_flux = ec_flux_flops(d)
            wave = 40
            flux_fac = 2 * prim + pair_flux + wave + nc * (2 * d + 3) + nc
            flops_B = ((nq + nf) * prim + nf * flux_fac + pairs * pair_flux
                       + S_inc * (d + nc * (2 * d + 2) + 2 * nc)
                       + nfp * (pair_flux + d + nc * (2 * d + 3))
                       + nc * 2 * nnzR + nq * nc + nc * (nV_B * vf + mf) + nq * nc)
        else:
            pair_flux = 2 + d
            flops_B = (nf * (pair_flux + 2 * d + 4) + pairs * pair_flux
                       + S_inc * (d + 2 * d + 2 + 2) + nfp * (pair_flux + d + 2 * d + 3)
                       + 2 * nnzR + nq + nV_B * vf + mf + nq)
        bytes_B = f8 * (nq * nc + 2 * nf * nc + d * d * nq + d * ra.reference_element.num_faces * nq
                        + 2 * d * nf + nf + nq + np_ * nc) + 4.0 * nf + mb
    else:
        nnzD = sum(D.nnz for D in host.D)
        phys = (d + 2) * d * 2 if euler else d
        flops_B = (nq * phys + nf * (4 * d + 10) * nc
                   + d * d * nc * (2 * nq + 4 * nnzD / d)
                   + d * nc * (2 * nnzR + 2 * nf) + nc * nf + nc * 2 * nnzR + nc * nq
                   + nc * (nV_B * vf + mf) + nq * nc)
        bytes_B = f8 * (nq * nc + 2 * nf * nc + d * d * nq + d * nf + nf + nq + np_ * nc) + 4.0 * nf + mb
    bytes_stage = f8 * 5 * np_ * nc
    return Work(float(flops_A), float(flops_B), bytes_A, bytes_B, bytes_stage)


def one_kernel_bytes(host) -> float:
    """Algorithmic HBM bytes per element of the one-kernel StandardForm
    residual (std_compact_kernel): the element's modal state and its
    neighbours' (one per face), halfWLambda, the facet normals, BJf and mapP,
    the dense mass operator, and the residual written; no nodal states."""
    ra = host.sd.reference_approximation
    d, nc, nq, nf, np_ = ra.d, host.N_c, host.N_q, host.N_f, host.N_p
    nfac = ra.reference_element.num_faces
    mb = 8.0 * np_ * np_ if ra.V is not None else 0.0
    return 8.0 * (np_ * nc * (1 + nfac) + d * d * nq + d * nf + nf + np_ * nc) + 4.0 * nf + mb


def _unique_pairs(host) -> int:
    seen = set()
    for S in host.S:
        for j in range(S.n):
            for q in range(S.colptr[j] - 1, S.colptr[j + 1] - 1):
                i = S.rowval[q] - 1
                if i < j:
                    seen.add((i, j))
    return len(seen)


def geometric_factors_flops(d: int, metrics: str, n_map: int, n_q: int, n_f: int,
                            num_faces: int, n_curl: int = 0, project: bool = False) -> float:
    """FP64 flops per element of GeometricFactors as sse_geometric_factors
    evaluates it (mesh.jl:229-282, 284-339, 410-506): dense matrix-vector
    products at 2 flops per entry, the per-node metric algebra and the
    normals (3 products and 2 sums per component, one square root)."""
    normals = n_q * num_faces * d * (2 * d - 1) + n_f * (d * (2 * d - 1) + 2 * d)
    if metrics == "Exact":
        adj = 12 * 3 + 5 if d == 3 else 3
        work = (2.0 * d * d * n_map * n_map + 2.0 * d * d * n_map * (n_q + n_f)
                + adj * (n_q + n_f))
        if project:
            work += 2.0 * n_q * n_q
        return work + normals
    if d == 2:
        return (2.0 * 4 * n_map * n_map + 7 * n_map + 2.0 * 5 * n_q * n_map
                + 2.0 * 4 * n_f * n_map + normals)
    n1 = n_curl
    return (2.0 * 9 * n_map * n_map + 17 * n_map + 2.0 * 3 * n1 * n_map + 2.0 * 9 * n1 * n1
            + 9 * n1 + 2.0 * 18 * n1 * n1 + 9 * n1 + 2.0 * n_q * n_map
            + 2.0 * 9 * (n_q + n_f) * n1 + normals)
