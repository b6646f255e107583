"""Reference-element operators for tensor-product (collapsed-coordinate) SBP
approximations on triangles and tetrahedra.

Host-side FP64 restatement of ``ReferenceApproximation`` for
``ModalTensor``/``NodalTensor`` on ``Tri``/``Tet``
(src/SpatialDiscretizations/tensor_simplex.jl:142-306), its
``RefElemData`` (src/SpatialDiscretizations/ref_elem_data.jl:1-134) and the
collapsed quadrature rules (src/SpatialDiscretizations/quadrature_rules.jl:
76-166).  Array layouts follow the reference (Julia column-major): the
volume node index is sigma_out = M2*M3*(i1-1) + M3*(i2-1) + i3, i.e. eta_1
slowest and eta_d fastest, and a Kronecker product ``A (x) B`` acts with B on
the fast index, which is numpy's ``np.kron`` convention as well.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import polynomials as P


@dataclass(frozen=True)
class GaussRule:
    """``GaussQuadrature(q, a, b)`` (quadrature_rules.jl:9-13)."""
    q: int
    a: int = 0
    b: int = 0

    def nodes_weights(self):
        return P.gauss_jacobi(self.q + 1, self.a, self.b)


def LGQuadrature(q: int) -> GaussRule:
    return GaussRule(q, 0, 0)


@dataclass
class WarpedProduct:
    """Factors of ``WarpedTensorProductMap2D/3D`` (warped_product_2d.jl:2-23,
    warped_product_3d.jl:2-36) built as in tensor_simplex.jl:84-140.

    ``A`` is (M1, p+1); ``B`` is (M2, p+1, p+1); ``C`` is (M3, p+1, p+1, p+1)
    (3-D only).  ``sigma_in[i, j(, k)]`` is the 0-based modal index or -1;
    ``sigma_out`` the 0-based nodal index.
    """
    d: int
    p: int
    A: np.ndarray
    B: np.ndarray
    C: np.ndarray | None
    sigma_in: np.ndarray
    sigma_out: np.ndarray

    def dense(self) -> np.ndarray:
        p = self.p
        if self.d == 2:
            M1, M2 = self.A.shape[0], self.B.shape[0]
            V = np.zeros((M1 * M2, (p + 1) * (p + 2) // 2))
            for i in range(p + 1):
                for j in range(p + 1 - i):
                    col = self.sigma_in[i, j]
                    V[:, col] = np.kron(self.A[:, i], self.B[:, i, j])
            return V
        M1, M2, M3 = self.A.shape[0], self.B.shape[0], self.C.shape[0]
        V = np.zeros((M1 * M2 * M3, (p + 1) * (p + 2) * (p + 3) // 6))
        for i in range(p + 1):
            for j in range(p + 1 - i):
                for k in range(p + 1 - i - j):
                    col = self.sigma_in[i, j, k]
                    V[:, col] = np.kron(np.kron(self.A[:, i], self.B[:, i, j]),
                                        self.C[:, i, j, k])
            # noqa
        return V


def warped_product(d: int, p: int, eta: tuple) -> WarpedProduct:
    """tensor_simplex.jl:84-140 (orthonormal Dubiner basis in collapsed form)."""
    sq2 = math.sqrt(2.0)
    M = [len(e) for e in eta]
    A = np.zeros((M[0], p + 1))
    B = np.zeros((M[1], p + 1, p + 1))
    for i in range(p + 1):
        A[:, i] = sq2 * P.jacobi_p(eta[0], 0, 0, i)
        for j in range(p + 1 - i):
            B[:, i, j] = (1.0 - eta[1]) ** i * P.jacobi_p(eta[1], 2 * i + 1, 0, j)
    if d == 2:
        sigma_in = -np.ones((p + 1, p + 1), dtype=np.int64)
        l = 0
        for i in range(p + 1):
            for j in range(p + 1 - i):
                sigma_in[i, j] = l
                l += 1
        sigma_out = np.arange(M[0] * M[1], dtype=np.int64).reshape(M[0], M[1])
        return WarpedProduct(2, p, A, B, None, sigma_in, sigma_out)
    C = np.zeros((M[2], p + 1, p + 1, p + 1))
    sigma_in = -np.ones((p + 1, p + 1, p + 1), dtype=np.int64)
    l = 0
    for i in range(p + 1):
        for j in range(p + 1 - i):
            for k in range(p + 1 - i - j):
                sigma_in[i, j, k] = l
                l += 1
                C[:, i, j, k] = 2.0 * (1.0 - eta[2]) ** (i + j) * P.jacobi_p(
                    eta[2], 2 * i + 2 * j + 2, 0, k)
    sigma_out = np.arange(M[0] * M[1] * M[2], dtype=np.int64).reshape(M[0], M[1], M[2])
    return WarpedProduct(3, p, A, B, C, sigma_in, sigma_out)


def _lagrange_interp(src_nodes: np.ndarray, dst_nodes: np.ndarray) -> np.ndarray:
    """vandermonde(Line(), q, dst) / V_1D (tensor_simplex.jl:149-152)."""
    q = len(src_nodes) - 1
    V = P.vandermonde_1d(q, src_nodes)
    return np.linalg.solve(V.T, P.vandermonde_1d(q, dst_nodes).T).T


@dataclass
class RefElem:
    """Mapping data of StartUpDG ``RefElemData`` restated in
    ref_elem_data.jl:1-134 (degree-N mapping nodes, their derivative
    matrices, interpolation to volume and facet quadrature nodes, facet
    normals scaled by the reference facet Jacobian)."""
    shape: str
    N: int
    rst: tuple          # mapping nodes
    VDM: np.ndarray
    Drst: tuple         # derivative matrices at the mapping nodes
    rstq: tuple
    wq: np.ndarray
    Vq: np.ndarray      # mapping basis -> volume quadrature nodes
    rstf: tuple
    wf: np.ndarray
    Vf: np.ndarray      # mapping basis -> facet quadrature nodes
    nrstJ: tuple
    num_faces: int


@dataclass
class ReferenceApproximation:
    """``ReferenceApproximation`` (SpatialDiscretizations.jl:191-251)."""
    approx_type: str            # "ModalTensor" or "NodalTensor"
    shape: str                  # "Tri" or "Tet"
    p: int
    d: int
    N_p: int
    N_q: int
    N_f: int
    n1d: tuple                  # (M1, M2[, M3]) 1-D quadrature sizes
    eta_1d: tuple
    D_1d: tuple
    R_L: tuple                  # (1, n) rows
    R_R: tuple
    facet_interp: dict          # named 1-D interpolation factors
    D: tuple                    # dense N_q x N_q derivative operators (collapsed)
    V: np.ndarray | None        # dense N_q x N_p (None for NodalTensor: identity)
    warped: WarpedProduct | None
    R: np.ndarray               # dense N_f x N_q
    W: np.ndarray               # N_q
    B: np.ndarray               # N_f
    J_ref: np.ndarray
    Lambda_ref: np.ndarray      # N_q x d x d
    reference_element: RefElem
    nodes_per_face: int = field(default=0)

    @property
    def V_dense(self) -> np.ndarray:
        return np.eye(self.N_q) if self.V is None else self.V


def _meshgrid_flat(*axes):
    """Flattened tensor grid with the first axis slowest (quadrature_rules.jl:
    343-352 followed by ``[:]``)."""
    grids = np.meshgrid(*axes, indexing="ij")
    return [g.reshape(-1) for g in grids]


def chi_tri(e1, e2):
    """Duffy map square -> triangle (tensor_simplex.jl:2-4)."""
    return 0.5 * (1.0 + e1) * (1.0 - e2) - 1.0, e2


def chi_tet(e1, e2, e3):
    """Duffy map cube -> tetrahedron (tensor_simplex.jl:7-11)."""
    xi_pri1 = 0.5 * (1.0 + e1) * (1.0 - e3) - 1.0
    xi_pyr2 = 0.5 * (1.0 + e2) * (1.0 - e3) - 1.0
    return 0.5 * (1.0 + xi_pri1) * (1.0 - e2) - 1.0, xi_pyr2, e3


def reference_geometric_factors(shape: str, rules: tuple, eta: tuple):
    """tensor_simplex.jl:13-82: J_ref and Lambda_ref[:, l, m] = J d eta_l / d xi_m."""
    if shape == "Tri":
        e1, e2 = _meshgrid_flat(*eta)
        N = e1.size
        L = np.zeros((N, 2, 2))
        ab = [(r.a, r.b) for r in rules]
        if ab == [(0, 0), (0, 0)]:
            J = 0.5 * (1.0 - e2)
            L[:, 0, 0] = 1.0
            L[:, 0, 1] = 0.5 * (1.0 + e1)
            L[:, 1, 1] = 0.5 * (1.0 - e2)
        elif ab == [(0, 0), (1, 0)]:
            J = 0.5 * np.ones(N)
            L[:, 0, 0] = 1.0 / (1.0 - e2)
            L[:, 0, 1] = 0.5 * (1.0 + e1) * (1.0 / (1.0 - e2))
            L[:, 1, 1] = 0.5 * np.ones(N)
        else:
            raise ValueError("Chosen Jacobi weight not supported")
        return J, L
    e1, e2, e3 = _meshgrid_flat(*eta)
    N = e1.size
    L = np.zeros((N, 3, 3))
    ab = [(r.a, r.b) for r in rules]
    if ab == [(0, 0), (0, 0), (0, 0)]:
        J = 0.5 * (1.0 - e2) * (0.5 * (1.0 - e3)) ** 2
        L[:, 0, 0] = 0.5 * (1.0 - e3)
        L[:, 0, 1] = 0.5 * (1.0 + e1) * (0.5 * (1.0 - e3))
        L[:, 0, 2] = 0.5 * (1.0 + e1) * (0.5 * (1.0 - e3))
        L[:, 1, 1] = 0.5 * (1.0 - e2) * (0.5 * (1.0 - e3))
        L[:, 1, 2] = 0.5 * (1.0 + e2) * (0.5 * (1.0 - e2)) * (0.5 * (1.0 - e3))
        L[:, 2, 2] = 0.5 * (1.0 - e2) * (0.5 * (1.0 - e3)) ** 2
    elif ab == [(0, 0), (0, 0), (1, 0)]:
        J = 0.125 * (1.0 - e2) * (1.0 - e3)
        L[:, 0, 0] = 0.5 * np.ones(N)
        L[:, 0, 1] = 0.25 * (1.0 + e1)
        L[:, 0, 2] = 0.25 * (1.0 + e1)
        L[:, 1, 1] = 0.25 * (1.0 - e2)
        L[:, 1, 2] = 0.125 * (1.0 + e2) * (1.0 - e2)
        L[:, 2, 2] = 0.125 * (1.0 - e2) * (1.0 - e3)
    else:
        raise ValueError("Chosen Jacobi weight not supported")
    return J, L


def _simplex_basis(shape, N, *rst):
    if shape == "Tri":
        V, Vr, Vs = P.tri_basis(N, *rst)
        return V, (Vr, Vs)
    V, Vr, Vs, Vt = P.tet_basis(N, *rst)
    return V, (Vr, Vs, Vt)


# mapping nodes of the tetrahedron: Warburton's warp-and-blend set (the
# counterpart of the triangle's), or "equispaced"
TET_MAPPING_NODES = "warp_blend"


def simplex_nodes(shape: str, N: int):
    return P.tri_nodes(N) if shape == "Tri" else P.tet_nodes(N, TET_MAPPING_NODES)


def _ref_elem(shape: str, N: int, rstq, wq, rstf, wf, nrstJ, num_faces) -> RefElem:
    rst = simplex_nodes(shape, N)
    VDM, grads = _simplex_basis(shape, N, *rst)
    Drst = tuple(np.linalg.solve(VDM.T, G.T).T for G in grads)
    Vq = np.linalg.solve(VDM.T, _simplex_basis(shape, N, *rstq)[0].T).T
    Vf = np.linalg.solve(VDM.T, _simplex_basis(shape, N, *rstf)[0].T).T
    return RefElem(shape, N, rst, VDM, Drst, rstq, wq, Vq, rstf, wf, Vf, nrstJ, num_faces)


def _collapsed_quadrature(shape: str, rules: tuple):
    """``quadrature(::Tri|::Tet, NTuple of line rules)`` (quadrature_rules.jl:
    131-166): the tensor grid of the 1-D rules (first rule slowest) mapped by
    the collapsed-coordinate map, with the weights of the rules' Jacobi
    parameters."""
    eta = [r.nodes_weights() for r in rules]
    ab = [(r.a, r.b) for r in rules]
    if shape == "Tri":
        g1, g2 = _meshgrid_flat(eta[0][0], eta[1][0])
        w = np.multiply(*_meshgrid_flat(eta[0][1], eta[1][1]))
        if ab == [(0, 0), (0, 0)]:
            w = 0.5 * (1.0 - g2) * w
        elif ab == [(0, 0), (1, 0)]:
            w = 0.5 * w
        else:
            raise ValueError("Chosen Jacobi weight not supported")
        return chi_tri(g1, g2), w
    g1, g2, g3 = _meshgrid_flat(eta[0][0], eta[1][0], eta[2][0])
    w = np.prod(_meshgrid_flat(eta[0][1], eta[1][1], eta[2][1]), axis=0)
    if ab == [(0, 0), (0, 0), (0, 0)]:
        w = 0.125 * (1.0 - g2) * (1.0 - g3) ** 2 * w
    elif ab == [(0, 0), (0, 0), (1, 0)]:
        w = 0.125 * (1.0 - g2) * (1.0 - g3) * w
    else:
        raise ValueError("Chosen Jacobi weight not supported")
    return chi_tet(g1, g2, g3), w


def _facet_nodes(shape: str, facet_rule):
    """Facet quadrature nodes, weights and scaled reference normals of the
    reference element (ref_elem_data.jl:22-27 for the triangle's edges; the
    tetrahedron's four faces from a triangle rule)."""
    if shape == "Tri":
        eta_f, w_f1 = facet_rule.nodes_weights()
        nf1 = len(eta_f)
        rf = np.concatenate([eta_f, -eta_f, -np.ones(nf1)])
        sf = np.concatenate([-np.ones(nf1), eta_f, eta_f])
        nrJ = np.concatenate([np.zeros(nf1), np.ones(nf1), -np.ones(nf1)])
        nsJ = np.concatenate([-np.ones(nf1), np.ones(nf1), np.zeros(nf1)])
        return (rf, sf), np.concatenate([w_f1, w_f1, w_f1]), (nrJ, nsJ), 3
    (r2, s2), w_2d = _collapsed_quadrature("Tri", facet_rule)
    ee = np.ones_like(r2)
    zz = np.zeros_like(r2)
    rf = np.concatenate([r2, -(ee + r2 + s2), -ee, r2])
    sf = np.concatenate([-ee, r2, r2, s2])
    tf = np.concatenate([s2, s2, s2, -ee])
    nrJ = np.concatenate([zz, ee, -ee, zz])
    nsJ = np.concatenate([-ee, ee, zz, zz])
    ntJ = np.concatenate([zz, ee, zz, -ee])
    return (rf, sf, tf), np.concatenate([w_2d] * 4), (nrJ, nsJ, ntJ), 4


def _multidimensional(approx_type: str, shape: str, p: int, mapping_degree: int,
                      volume_quadrature_rule, facet_quadrature_rule) -> ReferenceApproximation:
    """``ReferenceApproximation(ModalMulti(p)|NodalMulti(p), Tri()|Tet();
    mapping_degree, volume_quadrature_rule, facet_quadrature_rule)``
    (multidimensional.jl:1-76): the orthonormal simplex basis VDM and its
    gradients at the volume nodes, the projection P = (VDM' W VDM)^-1 VDM' W,
    D_m = grad_m VDM P, R = Vf P; V = VDM (ModalMulti, dense) or the identity
    (NodalMulti).  No reference mapping (the metric terms apply directly).

    The reference's default rules (``DefaultQuadrature(2p)``: tabulated
    Xiao-Gimbutas / Jaskowiec-Sukumar nodes from third-party packages) are
    not restated here; collapsed tensor-product rules (tuples of Gauss line
    rules, quadrature_rules.jl:131-166) are, and the triangle's facet rule
    defaults to the Gauss rule of DefaultQuadrature(2p) on a line (p + 1
    points)."""
    d = 2 if shape == "Tri" else 3
    if volume_quadrature_rule is None:
        raise ValueError(f"{approx_type}: pass volume_quadrature_rule as a tuple of {d} line rules "
                         "(the tabulated default rules are not available)")
    if facet_quadrature_rule is None:
        if d == 3:
            raise ValueError(f"{approx_type} on Tet: pass facet_quadrature_rule as a tuple of 2 line rules")
        facet_quadrature_rule = LGQuadrature(p)
    (rq, wq) = _collapsed_quadrature(shape, tuple(volume_quadrature_rule))
    rstf, wf, nrstJ, nfaces = _facet_nodes(shape, facet_quadrature_rule)
    ref = _ref_elem(shape, mapping_degree, rq, wq, rstf, wf, nrstJ, nfaces)
    VDM, grads = _simplex_basis(shape, p, *rq)
    Vf = _simplex_basis(shape, p, *rstf)[0]
    Pq = np.linalg.solve(VDM.T @ (wq[:, None] * VDM), VDM.T * wq[None, :])
    D = tuple(G @ Pq for G in grads)
    R = Vf @ Pq
    N_q = len(wq)
    V = VDM if approx_type == "ModalMulti" else None
    N_p = VDM.shape[1] if V is not None else N_q
    L_ref = np.zeros((N_q, d, d))
    for m in range(d):
        L_ref[:, m, m] = 1.0
    return ReferenceApproximation(
        approx_type=approx_type, shape=shape, p=p, d=d, N_p=N_p, N_q=N_q, N_f=R.shape[0],
        n1d=(), eta_1d=(), D_1d=(), R_L=(), R_R=(), facet_interp={}, D=D, V=V, warped=None,
        R=R, W=ref.wq.copy(), B=ref.wf.copy(), J_ref=np.ones(N_q), Lambda_ref=L_ref,
        reference_element=ref, nodes_per_face=R.shape[0] // nfaces)


def reference_approximation(approx_type: str, shape: str, p: int,
                            mapping_degree: int = 1, volume_quadrature_rule=None,
                            facet_quadrature_rule=None) -> ReferenceApproximation:
    """``ReferenceApproximation(ModalTensor(p)|NodalTensor(p), Tri()|Tet();
    mapping_degree)`` with the default quadrature rules
    (tensor_simplex.jl:158-306), or ``ModalMulti(p)|NodalMulti(p)`` with
    collapsed tensor-product rules (multidimensional.jl:1-76)."""
    if approx_type in ("ModalMulti", "NodalMulti"):
        if shape not in ("Tri", "Tet"):
            raise ValueError(f"unsupported element {shape}")
        return _multidimensional(approx_type, shape, p, mapping_degree, volume_quadrature_rule,
                                 facet_quadrature_rule)
    if approx_type not in ("ModalTensor", "NodalTensor"):
        raise ValueError(f"unsupported approximation type {approx_type}")
    if shape == "Tri":
        vol_rules = (LGQuadrature(p), LGQuadrature(p))
        fac_rule = LGQuadrature(p)
        d = 2
    elif shape == "Tet":
        vol_rules = (LGQuadrature(p), LGQuadrature(p), GaussRule(p, 1, 0))
        fac_rules = (LGQuadrature(p), GaussRule(p, 1, 0))
        d = 3
    else:
        raise ValueError(f"unsupported element {shape}")

    # operators_1d (tensor_simplex.jl:142-156)
    eta, wts, D1, RL, RR = [], [], [], [], []
    for rule in vol_rules:
        x, w = rule.nodes_weights()
        q = len(x) - 1
        V1 = P.vandermonde_1d(q, x)
        eta.append(x)
        wts.append(w)
        D1.append(np.linalg.solve(V1.T, P.grad_vandermonde_1d(q, x).T).T)
        RL.append(np.linalg.solve(V1.T, P.vandermonde_1d(q, np.array([-1.0])).T).T)
        RR.append(np.linalg.solve(V1.T, P.vandermonde_1d(q, np.array([1.0])).T).T)
    n1d = tuple(len(e) for e in eta)
    J_ref, L_ref = reference_geometric_factors(shape, vol_rules, tuple(eta))
    I = [np.eye(n) for n in n1d]

    if shape == "Tri":
        eta_f, w_f1 = fac_rule.nodes_weights()
        e1_to_f = I[0] if vol_rules[0] == fac_rule else _lagrange_interp(eta[0], eta_f)
        e2_to_f = I[1] if vol_rules[1] == fac_rule else _lagrange_interp(eta[1], eta_f)
        R = np.vstack([np.kron(e1_to_f, RL[1]), np.kron(RR[0], e2_to_f),
                       np.kron(RL[0], e2_to_f)])
        D = (np.kron(D1[0], I[1]), np.kron(I[0], D1[1]))
        # volume quadrature (quadrature_rules.jl:125-141)
        g1, g2 = _meshgrid_flat(eta[0], eta[1])
        w2 = np.multiply(*_meshgrid_flat(wts[0], wts[1]))
        rq, sq = chi_tri(g1, g2)
        wq = 0.5 * (1.0 - g2) * w2
        # facets (ref_elem_data.jl:22-27)
        wf = np.concatenate([w_f1, w_f1, w_f1])
        nf1 = len(eta_f)
        rf = np.concatenate([eta_f, -eta_f, -np.ones(nf1)])
        sf = np.concatenate([-np.ones(nf1), eta_f, eta_f])
        nrJ = np.concatenate([np.zeros(nf1), np.ones(nf1), -np.ones(nf1)])
        nsJ = np.concatenate([-np.ones(nf1), np.ones(nf1), np.zeros(nf1)])
        ref = _ref_elem("Tri", mapping_degree, (rq, sq), wq, (rf, sf), wf, (nrJ, nsJ), 3)
        interp = {"eta1_to_etaf": e1_to_f, "eta2_to_etaf": e2_to_f}
    else:
        ef1, wf1 = fac_rules[0].nodes_weights()
        ef2, wf2 = fac_rules[1].nodes_weights()
        e1_to_f1 = I[0] if vol_rules[0] == fac_rules[0] else _lagrange_interp(eta[0], ef1)
        e2_to_f1 = I[1] if vol_rules[1] == fac_rules[0] else _lagrange_interp(eta[1], ef1)
        e2_to_f2 = I[1] if vol_rules[1] == fac_rules[1] else _lagrange_interp(eta[1], ef2)
        e3_to_f2 = I[2] if vol_rules[2] == fac_rules[1] else _lagrange_interp(eta[2], ef2)
        kr = lambda a, b, c: np.kron(np.kron(a, b), c)
        R = np.vstack([kr(e1_to_f1, RL[1], e3_to_f2), kr(RR[0], e2_to_f1, e3_to_f2),
                       kr(RL[0], e2_to_f1, e3_to_f2), kr(e1_to_f1, e2_to_f2, RL[2])])
        D = (kr(D1[0], I[1], I[2]), kr(I[0], D1[1], I[2]), kr(I[0], I[1], D1[2]))
        g1, g2, g3 = _meshgrid_flat(eta[0], eta[1], eta[2])
        w3 = np.prod(_meshgrid_flat(wts[0], wts[1], wts[2]), axis=0)
        rq, sq, tq = chi_tet(g1, g2, g3)
        wq = 0.125 * (1.0 - g2) * (1.0 - g3) * w3     # (0,0),(0,0),(1,0) rule
        # facet rule: collapsed triangle (LG x GJ(1,0)) (ref_elem_data.jl:87-88, quadrature_rules.jl:125-141)
        a2, b2 = _meshgrid_flat(ef1, ef2)
        w2 = np.multiply(*_meshgrid_flat(wf1, wf2))
        r2, s2 = chi_tri(a2, b2)
        w_2d = 0.5 * w2
        ee = np.ones_like(r2)
        zz = np.zeros_like(r2)
        rf = np.concatenate([r2, -(ee + r2 + s2), -ee, r2])
        sf = np.concatenate([-ee, r2, r2, s2])
        tf = np.concatenate([s2, s2, s2, -ee])
        wf = np.concatenate([w_2d] * 4)
        nrJ = np.concatenate([zz, ee, -ee, zz])
        nsJ = np.concatenate([-ee, ee, zz, zz])
        ntJ = np.concatenate([zz, ee, zz, -ee])
        ref = _ref_elem("Tet", mapping_degree, (rq, sq, tq), wq, (rf, sf, tf), wf,
                        (nrJ, nsJ, ntJ), 4)
        interp = {"eta1_to_etaf1": e1_to_f1, "eta2_to_etaf1": e2_to_f1,
                  "eta2_to_etaf2": e2_to_f2, "eta3_to_etaf2": e3_to_f2}

    N_q = int(np.prod(n1d))
    if approx_type == "ModalTensor":
        wp = warped_product(d, p, tuple(eta))
        V = wp.dense()
    else:
        wp = None
        V = None
    N_p = V.shape[1] if V is not None else N_q
    N_f = R.shape[0]
    return ReferenceApproximation(
        approx_type=approx_type, shape=shape, p=p, d=d, N_p=N_p, N_q=N_q, N_f=N_f,
        n1d=n1d, eta_1d=tuple(eta), D_1d=tuple(D1), R_L=tuple(RL), R_R=tuple(RR),
        facet_interp=interp, D=D, V=V, warped=wp, R=R, W=ref.wq.copy(), B=ref.wf.copy(),
        J_ref=J_ref, Lambda_ref=L_ref, reference_element=ref,
        nodes_per_face=N_f // ref.num_faces)


def reference_derivative_operators(ra: ReferenceApproximation) -> tuple:
    """D_xi_m = sum_l diag(Lambda_ref[:, l, m] / J_ref) D_eta_l
    (SpatialDiscretizations.jl:414-418)."""
    out = []
    for m in range(ra.d):
        acc = np.zeros((ra.N_q, ra.N_q))
        for l in range(ra.d):
            acc = acc + (ra.Lambda_ref[:, l, m] / ra.J_ref)[:, None] * ra.D[l]
        out.append(acc)
    return tuple(out)


def check_sbp_property(ra: ReferenceApproximation) -> tuple:
    """max |W D_xi_m + D_xi_m^T W - R^T B diag(n_m) R| (SpatialDiscretizations.jl:441-455)."""
    Dxi = reference_derivative_operators(ra)
    W = np.diag(ra.W)
    out = []
    for m in range(ra.d):
        E = ra.R.T @ np.diag(ra.B * ra.reference_element.nrstJ[m]) @ ra.R
        out.append(float(np.abs(W @ Dxi[m] + Dxi[m].T @ W - E).max()))
    return tuple(out)
