"""Periodic uniform simplex meshes, curvilinear warping, face connectivity
and geometric factors.

Host-side FP64 restatement of src/SpatialDiscretizations/mesh.jl
(``uniform_periodic_mesh`` :133-179 and :508-525 including the collapsed
orientation of tetrahedra :150-170, ``warp_mesh`` :23-76,
``GeometricFactors`` exact :229-282 and conservative-curl :284-339, :410-506)
and of SpatialDiscretizations.jl:310-392 (``project_jacobian!``,
``SpatialDiscretization``).  Everything is vectorised over elements so that
the largest configurations (tens of thousands of curved tetrahedra) build in
seconds.  Array layouts are the reference's column-major ones stored as
C-order numpy arrays with the axes reversed, i.e. a Julia array of size
(N_q, d, d, N_e) is held as numpy shape (N_e, d, d, N_q) -- the memory
layout is identical, so buffers pass through the C-ABI unchanged.
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np

from . import polynomials as P
from .reference import ReferenceApproximation, simplex_nodes, _simplex_basis


# ---------------------------------------------------------------------------
# Uniform meshes
# ---------------------------------------------------------------------------

def _grid_vertices(M, limits):
    """Vertices of a tensor grid, first coordinate fastest (StartUpDG
    ``uniform_mesh`` numbering), mapped from [-1, 1]^d onto ``limits`` as in
    mesh.jl:172-175."""
    axes = [np.linspace(-1.0, 1.0, m + 1) for m in M]
    grids = np.meshgrid(*axes[::-1], indexing="ij")[::-1]
    V = [g.reshape(-1) for g in grids]
    return [limits[m][0] + 0.5 * (limits[m][1] - limits[m][0]) * (V[m] + 1.0)
            for m in range(len(M))]


def uniform_tri_elements(Mx: int, My: int) -> np.ndarray:
    """Two triangles per cell of an Mx x My grid with corners
    v1=(i,j), v2=(i+1,j), v3=(i+1,j+1), v4=(i,j+1): (v1, v2, v3) and
    (v3, v4, v1), counter-clockwise, 0-based vertex ids, cells numbered with
    x fastest.  This is StartUpDG's ``uniform_mesh(Tri(), Kx, Ky)`` split
    and vertex order (which vertex is the collapsed one matters for
    ModalTensor); the reference's own goldens pin it (test/runtests.jl:57,
    :114-119 are reproduced to round-off with it and not with the other
    diagonal or rotations)."""
    nx = Mx + 1
    ex, ey = np.meshgrid(np.arange(Mx), np.arange(My), indexing="xy")
    ex = ex.reshape(-1)
    ey = ey.reshape(-1)
    v1 = ex + ey * nx
    v2 = v1 + 1
    v3 = v1 + 1 + nx
    v4 = v1 + nx
    t1 = np.stack([v1, v2, v3], axis=1)
    t2 = np.stack([v3, v4, v1], axis=1)
    return np.stack([t1, t2], axis=1).reshape(-1, 3)


def uniform_tet_elements(Mx: int, My: int, Mz: int) -> np.ndarray:
    """Six tetrahedra per hexahedral cell (Kuhn split along the cell's main
    diagonal), conforming across cells; 0-based vertex ids."""
    nx, ny = Mx + 1, My + 1
    vid = lambda i, j, k: i + nx * (j + ny * k)
    ci, cj, ck = np.meshgrid(np.arange(Mx), np.arange(My), np.arange(Mz), indexing="ij")
    ci = ci.transpose(2, 1, 0).reshape(-1)
    cj = cj.transpose(2, 1, 0).reshape(-1)
    ck = ck.transpose(2, 1, 0).reshape(-1)
    perms = [(0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)]
    tets = []
    for perm in perms:
        off = np.zeros(3, dtype=np.int64)
        verts = [vid(ci, cj, ck)]
        for ax in perm:
            off[ax] += 1
            verts.append(vid(ci + off[0], cj + off[1], ck + off[2]))
        tets.append(np.stack(verts, axis=1))
    return np.stack(tets, axis=1).reshape(-1, 4)


def collapsed_orientation(EToV: np.ndarray, VXYZ) -> np.ndarray:
    """mesh.jl:150-170: sort each tetrahedron's vertices by descending global
    id, then swap the first two if the resulting orientation is negative, so
    that both neighbours see a shared face with the same vertex order and
    the collapsed facet quadrature nodes coincide."""
    E = -np.sort(-EToV, axis=1)
    X = np.stack([np.stack([VXYZ[m][E[:, c]] - VXYZ[m][E[:, 0]] for m in range(3)], axis=1)
                  for c in (1, 2, 3)], axis=2)          # (N_e, 3, 3) columns = edges
    det = np.linalg.det(X)
    out = E.copy()
    neg = det < 0
    out[neg, 0] = E[neg, 1]
    out[neg, 1] = E[neg, 0]
    return out


# ---------------------------------------------------------------------------
# Mesh data
# ---------------------------------------------------------------------------

@dataclass
class MeshData:
    """Physical node positions and connectivity (StartUpDG ``MeshData``
    fields used by the reference: xyz, xyzq, xyzf, mapP).

    ``xyz[m]`` is (N_e, N_map); ``xyzq[m]`` is (N_e, N_q); ``xyzf[m]`` is
    (N_e, N_f); ``mapP`` is (N_e, N_f) holding 1-based linear indices into the
    column-major (N_f, N_e) facet array, as the reference's ``mesh.mapP``.
    """
    d: int
    VXYZ: list
    EToV: np.ndarray
    xyz: list
    xyzq: list
    xyzf: list
    mapP: np.ndarray
    limits: tuple

    @property
    def N_e(self) -> int:
        return self.EToV.shape[0]


def _barycentric_map(shape, rst, VXYZ, EToV):
    """Affine map of each element (StartUpDG x = V1 * VX[EToV]')."""
    if shape == "Tri":
        r, s = rst
        lam = [-(r + s) / 2.0, (1.0 + r) / 2.0, (1.0 + s) / 2.0]
    else:
        r, s, t = rst
        lam = [-(1.0 + r + s + t) / 2.0, (1.0 + r) / 2.0, (1.0 + s) / 2.0, (1.0 + t) / 2.0]
    out = []
    for m in range(len(VXYZ)):
        vx = VXYZ[m][EToV]                       # (N_e, nverts)
        out.append(sum(vx[:, c:c + 1] * lam[c][None, :] for c in range(len(lam))))
    return out


def periodic_map_p(xyzf, limits, tol: float = 1.0e-9) -> np.ndarray:
    """Match every facet node with the coincident facet node of the
    neighbouring element, wrapping coordinates periodically (StartUpDG
    ``make_periodic``); returns the 1-based linear index into (N_f, N_e)."""
    N_e, N_f = xyzf[0].shape
    keys = []
    for m, x in enumerate(xyzf):
        lo, hi = limits[m]
        frac = (x.reshape(-1) - lo) / (hi - lo)
        q = np.rint(frac / tol).astype(np.int64)
        period = int(np.rint(1.0 / tol))
        keys.append(np.mod(q, period))
    keys = np.stack(keys, axis=1)
    order = np.lexsort(keys.T[::-1])
    ks = keys[order]
    same_next = np.all(ks[1:] == ks[:-1], axis=1)
    n = ks.shape[0]
    if n % 2 != 0 or not np.all(same_next[0::2]) or (n > 2 and np.any(same_next[1::2])):
        raise RuntimeError("facet nodes do not pair up: mesh is not conforming/periodic")
    a = order[0::2]
    b = order[1::2]
    partner = np.empty(n, dtype=np.int64)
    partner[a] = b
    partner[b] = a
    # flat index in numpy (N_e, N_f) C-order equals Julia's column-major (N_f, N_e)
    return (partner + 1).reshape(N_e, N_f)


def uniform_periodic_mesh(ra: ReferenceApproximation, limits, M) -> MeshData:
    """``uniform_periodic_mesh(reference_approximation, limits, M)``
    (mesh.jl:133-179, :508-541)."""
    ref = ra.reference_element
    d = ra.d
    VXYZ = _grid_vertices(M, limits)
    if ra.shape == "Tri":
        EToV = uniform_tri_elements(*M)
    else:
        EToV = collapsed_orientation(uniform_tet_elements(*M), VXYZ)
    xyz = _barycentric_map(ra.shape, ref.rst, VXYZ, EToV)
    xyzq = _barycentric_map(ra.shape, ref.rstq, VXYZ, EToV)
    xyzf = _barycentric_map(ra.shape, ref.rstf, VXYZ, EToV)
    mapP = periodic_map_p(xyzf, limits)
    return MeshData(d, VXYZ, EToV, xyz, xyzq, xyzf, mapP, tuple(limits))


def _with_positions(mesh: MeshData, ra: ReferenceApproximation, xyz) -> MeshData:
    ref = ra.reference_element
    xyzq = [x @ ref.Vq.T for x in xyz]
    xyzf = [x @ ref.Vf.T for x in xyz]
    return MeshData(mesh.d, mesh.VXYZ, mesh.EToV, xyz, xyzq, xyzf, mesh.mapP, mesh.limits)


def warp_mesh(mesh: MeshData, ra: ReferenceApproximation, kind: str, factor: float,
              L) -> MeshData:
    """``warp_mesh`` with ``DelReyWarping`` / ``ChanWarping`` (mesh.jl:30-76,
    :106-120) applied at the mapping nodes."""
    pi = np.pi
    if mesh.d == 2:
        x, y = mesh.xyz
        if kind == "DelRey":
            xn = x + L[0] * factor * np.sin(pi * x / L[0]) * np.sin(pi * y / L[1])
            yn = y + L[1] * factor * np.exp(1.0 - y / L[1]) * np.sin(pi * x / L[0]) * np.sin(pi * y / L[1])
        elif kind == "Chan":
            xn = x + L[0] * factor * np.cos(pi / L[0] * (x - 0.5 * L[0])) * np.cos(3 * pi / L[1] * (y - 0.5 * L[1]))
            yn = y + L[1] * factor * np.sin(4 * pi / L[0] * (xn - 0.5 * L[0])) * np.cos(pi / L[1] * (y - 0.5 * L[1]))
        else:
            raise ValueError(kind)
        return _with_positions(mesh, ra, [xn, yn])
    x, y, z = mesh.xyz
    if kind == "Chan":
        yn = y + L[1] * factor * np.cos(3 * pi / L[0] * (x - 0.5 * L[0])) * np.cos(pi / L[1] * (y - 0.5 * L[1])) * np.cos(pi / L[2] * (z - 0.5 * L[2]))
        xn = x + L[0] * factor * np.cos(pi / L[0] * (x - 0.5 * L[0])) * np.sin(4 * pi / L[1] * (yn - 0.5 * L[1])) * np.cos(pi / L[2] * (z - 0.5 * L[2]))
        zn = z + L[2] * factor * np.cos(pi / L[0] * (xn - 0.5 * L[0])) * np.cos(2 * pi / L[1] * (yn - 0.5 * L[1])) * np.cos(pi / L[2] * (z - 0.5 * L[2]))
    elif kind == "DelRey":
        xn = x + L[0] * factor * np.sin(pi * x / L[0]) * np.sin(pi * y / L[1])
        yn = y + L[1] * factor * np.exp((1.0 - y) / L[1]) * np.sin(pi * x / L[0]) * np.sin(pi * y / L[1])
        zn = z + 0.25 * L[2] * factor * (np.sin(2 * pi * x / L[0]) * np.sin(2 * pi * y / L[1])) * np.sin(2 * pi * z / L[2])
    else:
        raise ValueError(kind)
    return _with_positions(mesh, ra, [xn, yn, zn])


# ---------------------------------------------------------------------------
# Geometric factors
# ---------------------------------------------------------------------------

@dataclass
class GeometricFactors:
    """``GeometricFactors`` (SpatialDiscretizations.jl:283-289), numpy
    shapes with reversed axes: J_q (N_e, N_q); Lambda_q (N_e, d(n), d(m), N_q)
    holding Julia's Lambda_q[i, m, n, k] = J d xi_m / d x_n at [k, n, m, i];
    J_f (N_e, N_f); nJf (N_e, N_f, d); nJq (N_e, N_q, N_fac, d)."""
    J_q: np.ndarray
    Lambda_q: np.ndarray
    J_f: np.ndarray
    nJf: np.ndarray
    nJq: np.ndarray


def _normals(Lq_nm, Lf_nm, nrstJ, nodes_per_face, num_faces):
    """nJq[n, f, i] = sum_m Lambda_q[i, m, n] n_ref[m](f);
    nJf[m, i] = sum_n Lambda_f[i, n, m] nrstJ[n][i]; J_f = |nJf|
    (mesh.jl:262-279).  Lq_nm[k, n, m, i] = Lambda[i, m, n, k]."""
    d = len(nrstJ)
    N_e, _, _, N_q = Lq_nm.shape
    nJq = np.zeros((N_e, N_q, num_faces, d))
    for f in range(num_faces):
        nref = [nrstJ[m][nodes_per_face * f] for m in range(d)]
        for n in range(d):
            acc = Lq_nm[:, n, 0, :] * nref[0]
            for m in range(1, d):
                acc = acc + Lq_nm[:, n, m, :] * nref[m]
            nJq[:, :, f, n] = acc
    N_f = Lf_nm.shape[3]
    nJf = np.zeros((N_e, N_f, d))
    for m in range(d):
        # Lambda_f[i, n, m] -> Lf_nm[k, m, n, i]
        acc = Lf_nm[:, m, 0, :] * nrstJ[0][None, :]
        for n in range(1, d):
            acc = acc + Lf_nm[:, m, n, :] * nrstJ[n][None, :]
        nJf[:, :, m] = acc
    J_f = np.sqrt(np.sum(nJf ** 2, axis=2))
    return nJq, nJf, J_f


def _adjugate_3(A):
    """J * inv(A) for a stack of 3x3 matrices (the 3-D ``metrics``,
    mesh.jl:223-227), returning (J, Lambda) with Lambda = adj(A)."""
    a = A
    adj = np.empty_like(a)
    adj[..., 0, 0] = a[..., 1, 1] * a[..., 2, 2] - a[..., 1, 2] * a[..., 2, 1]
    adj[..., 0, 1] = a[..., 0, 2] * a[..., 2, 1] - a[..., 0, 1] * a[..., 2, 2]
    adj[..., 0, 2] = a[..., 0, 1] * a[..., 1, 2] - a[..., 0, 2] * a[..., 1, 1]
    adj[..., 1, 0] = a[..., 1, 2] * a[..., 2, 0] - a[..., 1, 0] * a[..., 2, 2]
    adj[..., 1, 1] = a[..., 0, 0] * a[..., 2, 2] - a[..., 0, 2] * a[..., 2, 0]
    adj[..., 1, 2] = a[..., 0, 2] * a[..., 1, 0] - a[..., 0, 0] * a[..., 1, 2]
    adj[..., 2, 0] = a[..., 1, 0] * a[..., 2, 1] - a[..., 1, 1] * a[..., 2, 0]
    adj[..., 2, 1] = a[..., 0, 1] * a[..., 2, 0] - a[..., 0, 0] * a[..., 2, 1]
    adj[..., 2, 2] = a[..., 0, 0] * a[..., 1, 1] - a[..., 0, 1] * a[..., 1, 0]
    J = a[..., 0, 0] * adj[..., 0, 0] + a[..., 0, 1] * adj[..., 1, 0] + a[..., 0, 2] * adj[..., 2, 0]
    return J, adj


def geometric_factors_exact(mesh: MeshData, ra: ReferenceApproximation) -> GeometricFactors:
    """``GeometricFactors(mesh, reference_element, ExactMetrics())``
    (mesh.jl:229-282): metrics from the exact derivatives of the degree-N
    mapping evaluated at the quadrature nodes."""
    ref = ra.reference_element
    d = ra.d
    # dxdr[k, i, m, n] = d x_m / d r_n at quadrature / facet nodes
    dq = np.stack([np.stack([(mesh.xyz[m] @ ref.Drst[n].T) @ ref.Vq.T for n in range(d)], axis=-1)
                   for m in range(d)], axis=-2)
    df = np.stack([np.stack([(mesh.xyz[m] @ ref.Drst[n].T) @ ref.Vf.T for n in range(d)], axis=-1)
                   for m in range(d)], axis=-2)
    if d == 2:
        def met(A):
            J = A[..., 0, 0] * A[..., 1, 1] - A[..., 0, 1] * A[..., 1, 0]
            L = np.empty_like(A)
            L[..., 0, 0] = A[..., 1, 1]
            L[..., 0, 1] = -A[..., 0, 1]
            L[..., 1, 0] = -A[..., 1, 0]
            L[..., 1, 1] = A[..., 0, 0]
            return J, L
    else:
        met = _adjugate_3
    J_q, Lq = met(dq)             # Lq[k, i, m, n] = Lambda[i, m, n]
    _, Lf = met(df)
    Lq_nm = Lq.transpose(0, 3, 2, 1)   # -> [k, n, m, i]
    Lf_nm = Lf.transpose(0, 3, 2, 1)
    nJq, nJf, J_f = _normals(Lq_nm, Lf_nm, ref.nrstJ, ra.nodes_per_face, ref.num_faces)
    return GeometricFactors(J_q, np.ascontiguousarray(Lq_nm), J_f, nJf, nJq)


def _curl_metrics_2d(x, y, Dr, Ds):
    """StartUpDG 2-D ``geometric_factors``: rxJ = y_s, sxJ = -y_r,
    ryJ = -x_s, syJ = x_r, J = x_r y_s - x_s y_r (values at mapping nodes)."""
    xr, xs = x @ Dr.T, x @ Ds.T
    yr, ys = y @ Dr.T, y @ Ds.T
    J = -xs * yr + xr * ys
    return ys, -yr, -xs, xr, J


def _curl_metrics_3d(x, y, z, Dr, Ds, Dt):
    """Conservative curl form of the 3-D metric terms (Kopriva 2006):
    (J grad xi_i)_n = - e_n . curl_xi(X_l grad_xi X_m), evaluated with
    nodal products and the nodal derivative matrices."""
    D = (Dr, Ds, Dt)
    d_ = lambda u, a: u @ D[a].T

    def curl_terms(a_, b_):
        # a_ is differentiated, b_ multiplies:  F_a = (D_a a_) * b_
        Fr, Fs, Ft = d_(a_, 0) * b_, d_(a_, 1) * b_, d_(a_, 2) * b_
        return (d_(Fs, 2) - d_(Ft, 1), d_(Ft, 0) - d_(Fr, 2), d_(Fr, 1) - d_(Fs, 0))

    rxJ, sxJ, txJ = curl_terms(y, z)
    ry, sy, ty = curl_terms(x, z)
    rz, sz, tz = curl_terms(y, x)
    ryJ, syJ, tyJ = -ry, -sy, -ty
    rzJ, szJ, tzJ = -rz, -sz, -tz
    return rxJ, sxJ, txJ, ryJ, syJ, tyJ, rzJ, szJ, tzJ


@dataclass
class MetricOperators:
    """Reference-element matrices the geometric factors are built from (the
    fields of ``sse_metric_operators``): derivative matrices at the mapping
    nodes, interpolation to the volume / facet quadrature nodes, the scaled
    reference normals, and for the tetrahedral curl metrics the degree N+1
    element of mesh.jl:414-433."""
    d: int
    metrics: str                 # "Exact" or "ChanWilcox"
    Drst: tuple
    Vq: np.ndarray
    Vf: np.ndarray
    nrstJ: tuple
    num_faces: int
    N_to_N1: np.ndarray | None = None
    D1: tuple | None = None
    Vq1: np.ndarray | None = None
    Vf1: np.ndarray | None = None
    project: np.ndarray | None = None


def metric_operators(ra: ReferenceApproximation, metrics: str = "Exact",
                     project_jac: bool = True) -> MetricOperators:
    """The matrices of ``metrics`` for ``ra``, built once per reference
    approximation and kept on it."""
    cache = ra.__dict__.setdefault("_metric_operators", {})
    key = (metrics, bool(project_jac))
    if key not in cache:
        cache[key] = _build_metric_operators(ra, metrics, project_jac)
    return cache[key]


def _build_metric_operators(ra: ReferenceApproximation, metrics: str,
                            project_jac: bool) -> MetricOperators:
    ref = ra.reference_element
    ops = MetricOperators(ra.d, metrics, tuple(ref.Drst), ref.Vq, ref.Vf, tuple(ref.nrstJ),
                          ref.num_faces)
    if metrics == "ChanWilcox" and ra.d == 3:
        N = ref.N
        r1, s1, t1 = simplex_nodes("Tet", N + 1)
        V1, G1 = _simplex_basis("Tet", N + 1, r1, s1, t1)
        ops.D1 = tuple(np.linalg.solve(V1.T, G.T).T for G in G1)
        ops.N_to_N1 = np.linalg.solve(ref.VDM.T, _simplex_basis("Tet", N, r1, s1, t1)[0].T).T
        N1_to_N = np.linalg.solve(V1.T, _simplex_basis("Tet", N + 1, *ref.rst)[0].T).T
        ops.Vq1 = ref.Vq @ N1_to_N
        ops.Vf1 = ref.Vf @ N1_to_N
    if metrics == "Exact" and project_jac:
        V = ra.V_dense
        W = np.diag(ra.W)
        ops.project = V @ np.linalg.inv(V.T @ W @ V) @ V.T @ W
    return ops


def geometric_factors_curl(mesh: MeshData, ra: ReferenceApproximation) -> GeometricFactors:
    """``GeometricFactors(..., ConservativeCurlMetrics())`` = ChanWilcoxMetrics
    (mesh.jl:284-339 for triangles, :410-506 for tetrahedra)."""
    ref = ra.reference_element
    d = ra.d
    N_e = mesh.N_e
    if d == 2:
        rxJ, sxJ, ryJ, syJ, J = _curl_metrics_2d(*mesh.xyz, *ref.Drst)
        Vq, Vf = ref.Vq, ref.Vf
        # Lambda[i, m, n]: (1,1)=rxJ (2,1)=sxJ (1,2)=ryJ (2,2)=syJ
        comp = {(0, 0): rxJ, (1, 0): sxJ, (0, 1): ryJ, (1, 1): syJ}
        J_q = J @ Vq.T
    else:
        mo = metric_operators(ra, "ChanWilcox")
        Vq, Vf = mo.Vq1, mo.Vf1
        x, y, z = mesh.xyz
        Dr, Ds, Dt = ref.Drst
        xr, xs, xt = x @ Dr.T, x @ Ds.T, x @ Dt.T
        yr, ys, yt = y @ Dr.T, y @ Ds.T, y @ Dt.T
        zr, zs, zt = z @ Dr.T, z @ Ds.T, z @ Dt.T
        J = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt)
        J_q = J @ ref.Vq.T
        N_to_N1 = mo.N_to_N1
        terms = _curl_metrics_3d(x @ N_to_N1.T, y @ N_to_N1.T, z @ N_to_N1.T, *mo.D1)
        rxJ, sxJ, txJ, ryJ, syJ, tyJ, rzJ, szJ, tzJ = terms
        comp = {(0, 0): rxJ, (1, 0): sxJ, (2, 0): txJ,
                (0, 1): ryJ, (1, 1): syJ, (2, 1): tyJ,
                (0, 2): rzJ, (1, 2): szJ, (2, 2): tzJ}
    N_q = Vq.shape[0]
    N_f = Vf.shape[0]
    Lq_nm = np.empty((N_e, d, d, N_q))
    Lf_nm = np.empty((N_e, d, d, N_f))
    for (m, n), val in comp.items():
        Lq_nm[:, n, m, :] = val @ Vq.T
        Lf_nm[:, n, m, :] = val @ Vf.T
    nJq, nJf, J_f = _normals(Lq_nm, Lf_nm, ref.nrstJ, ra.nodes_per_face, ref.num_faces)
    return GeometricFactors(J_q, Lq_nm, J_f, nJf, nJq)


def project_jacobian(J_q: np.ndarray, ra: ReferenceApproximation) -> np.ndarray:
    """project_jacobian! (SpatialDiscretizations.jl:310-317):
    J_q <- V (V^T W V)^{-1} V^T W J_q for every element."""
    return J_q @ metric_operators(ra, "Exact", True).project.T


@dataclass
class SpatialDiscretization:
    """``SpatialDiscretization`` (SpatialDiscretizations.jl:299-392)."""
    mesh: MeshData
    reference_approximation: ReferenceApproximation
    geometric_factors: GeometricFactors
    metrics: str

    @property
    def N_e(self) -> int:
        return self.mesh.N_e


def spatial_discretization(mesh: MeshData, ra: ReferenceApproximation,
                           metrics: str = "Exact", project_jac: bool = True,
                           geometry: str = "host") -> SpatialDiscretization:
    """``SpatialDiscretization(mesh, reference_approximation, metric_type;
    project_jacobian)``.  ``geometry="gpu"`` builds the geometric factors
    with the library's ``sse_geometric_factors`` (FP64, on the current CUDA
    device) instead of numpy."""
    if metrics == "ConservativeCurl":
        metrics = "ChanWilcox"
    if geometry == "gpu":
        from . import gb300
        gf = gb300.geometric_factors(mesh, ra, metrics, project_jac)
        return SpatialDiscretization(mesh, ra, gf, metrics)
    if geometry != "host":
        raise ValueError(geometry)
    if metrics == "Exact":
        gf = geometric_factors_exact(mesh, ra)
        if project_jac:
            gf.J_q = project_jacobian(gf.J_q, ra)
    elif metrics in ("ChanWilcox", "ConservativeCurl"):
        gf = geometric_factors_curl(mesh, ra)
        metrics = "ChanWilcox"
    else:
        raise ValueError(metrics)
    return SpatialDiscretization(mesh, ra, gf, metrics)


def check_normals(sd: SpatialDiscretization) -> float:
    """max |nJf[:, j, k] + nJf[:, mapP[j, k]]| (SpatialDiscretizations.jl:425-430)."""
    nJf = sd.geometric_factors.nJf.reshape(-1, sd.reference_approximation.d)
    idx = sd.mesh.mapP.reshape(-1) - 1
    return float(np.abs(nJf + nJf[idx]).max())


def check_facet_nodes(sd: SpatialDiscretization) -> float:
    """max |xyzf - xyzf[mapP]| up to periodic shifts (SpatialDiscretizations.jl:433-438)."""
    idx = sd.mesh.mapP.reshape(-1) - 1
    worst = 0.0
    for m, x in enumerate(sd.mesh.xyzf):
        lo, hi = sd.mesh.limits[m]
        L = hi - lo
        diff = x.reshape(-1) - x.reshape(-1)[idx]
        diff = diff - L * np.rint(diff / L)
        worst = max(worst, float(np.abs(diff).max()))
    return worst
