"""Orthogonal polynomials, Gauss-Jacobi rules and simplex interpolation nodes.

Host-side (numpy, FP64) restatement of the third-party numerics that the
reference's operator construction calls but does not vendor:

* Gauss-Jacobi nodes and weights (Jacobi.jl ``zgj``/``wgj``), used by
  ``quadrature(::Line, ::GaussQuadrature)`` in
  src/SpatialDiscretizations/quadrature_rules.jl:82-86.  Computed here by the
  Golub-Welsch eigenvalue method followed by Newton polishing on the
  three-term recurrence, with the classical closed-form weights.
* Orthonormal Jacobi polynomials ``jacobiP(x, a, b, n)`` (NodesAndModes.jl),
  called in src/SpatialDiscretizations/tensor_simplex.jl:97-98, 124-129,
  normalised to unit L2 norm against the weight (1-x)^a (1+x)^b.
* Orthonormal Proriol-Koornwinder-Dubiner bases on the reference triangle
  and tetrahedron with their gradients (StartUpDG ``basis``), written from
  the collapsed-coordinate product form and the chain rule.
* Warp-and-blend interpolation nodes on the triangle (Warburton 2006,
  J. Eng. Math. 56:247-262; Hesthaven & Warburton 2008, sec. 6.1), the
  degree-N mapping nodes that StartUpDG's ``RefElemData`` uses in
  src/SpatialDiscretizations/ref_elem_data.jl:11.
"""
from __future__ import annotations

import math

import numpy as np


# ---------------------------------------------------------------------------
# 1-D Jacobi polynomials
# ---------------------------------------------------------------------------

def jacobi_p(x, a: float, b: float, n: int) -> np.ndarray:
    """Orthonormal Jacobi polynomial P_n^{(a,b)} evaluated at ``x``.

    Normalised so that int_{-1}^{1} P_n^2 (1-x)^a (1+x)^b dx = 1, the
    convention of NodesAndModes ``jacobiP`` used by the reference's warped
    tensor-product Vandermonde (tensor_simplex.jl:97-98).  Three-term
    recurrence for the orthonormal family (Hesthaven & Warburton 2008,
    Appendix A).
    """
    x = np.asarray(x, dtype=np.float64)
    a = float(a)
    b = float(b)
    p0 = math.sqrt(2.0 ** (-(a + b + 1.0)) * math.gamma(a + b + 2.0)
                   / (math.gamma(a + 1.0) * math.gamma(b + 1.0)))
    pm1 = np.full_like(x, p0)
    if n == 0:
        return pm1
    p1 = ((a + b + 2.0) * x / 2.0 + (a - b) / 2.0) * math.sqrt(
        (a + b + 3.0) / ((a + 1.0) * (b + 1.0))) * p0
    if n == 1:
        return p1
    aold = 2.0 / (2.0 + a + b) * math.sqrt((a + 1.0) * (b + 1.0) / (a + b + 3.0))
    pcur = p1
    for i in range(1, n):
        h1 = 2.0 * i + a + b
        anew = 2.0 / (h1 + 2.0) * math.sqrt(
            (i + 1.0) * (i + 1.0 + a + b) * (i + 1.0 + a) * (i + 1.0 + b)
            / ((h1 + 1.0) * (h1 + 3.0)))
        bnew = -(a * a - b * b) / (h1 * (h1 + 2.0))
        pnext = (-aold * pm1 + (x - bnew) * pcur) / anew
        pm1, pcur = pcur, pnext
        aold = anew
    return pcur


def grad_jacobi_p(x, a: float, b: float, n: int) -> np.ndarray:
    """d/dx of the orthonormal Jacobi polynomial P_n^{(a,b)}."""
    x = np.asarray(x, dtype=np.float64)
    if n == 0:
        return np.zeros_like(x)
    return math.sqrt(n * (n + a + b + 1.0)) * jacobi_p(x, a + 1.0, b + 1.0, n - 1)


def _jacobi_p_std(x, a: float, b: float, n: int):
    """Classical (unnormalised) Jacobi P_n^{(a,b)} and its derivative."""
    x = np.asarray(x, dtype=np.float64)
    p_prev = np.ones_like(x)
    if n == 0:
        return p_prev, np.zeros_like(x)
    p = 0.5 * (a - b + (a + b + 2.0) * x)
    for k in range(2, n + 1):
        c1 = 2.0 * k * (k + a + b) * (2.0 * k + a + b - 2.0)
        c2 = (2.0 * k + a + b - 1.0) * (a * a - b * b)
        c3 = (2.0 * k + a + b - 2.0) * (2.0 * k + a + b - 1.0) * (2.0 * k + a + b)
        c4 = 2.0 * (k + a - 1.0) * (k + b - 1.0) * (2.0 * k + a + b)
        p_prev, p = p, ((c2 + c3 * x) * p - c4 * p_prev) / c1
    # derivative of the classical family: d/dx P_n = (n+a+b+1)/2 P_{n-1}^{(a+1,b+1)}
    dp = 0.5 * (n + a + b + 1.0) * _jacobi_p_std(x, a + 1.0, b + 1.0, n - 1)[0]
    return p, dp


def gauss_jacobi(q: int, a: float = 0.0, b: float = 0.0):
    """Gauss-Jacobi rule with ``q`` points for the weight (1-x)^a (1+x)^b.

    Returns ascending nodes and weights (Jacobi.jl ``zgj``/``wgj``, called by
    quadrature_rules.jl:82-86 with q = p + 1 points).
    """
    a = float(a)
    b = float(b)
    k = np.arange(q, dtype=np.float64)
    # Golub-Welsch: symmetric tridiagonal Jacobi matrix of the monic family
    diag = np.empty(q)
    for i in range(q):
        den = (2.0 * i + a + b) * (2.0 * i + a + b + 2.0)
        diag[i] = (b * b - a * a) / den if den != 0.0 else (b - a) / (a + b + 2.0)
    off = np.empty(max(q - 1, 0))
    for i in range(1, q):
        n = float(i)
        num = 4.0 * n * (n + a) * (n + b) * (n + a + b)
        den = (2.0 * n + a + b) ** 2 * (2.0 * n + a + b + 1.0) * (2.0 * n + a + b - 1.0)
        off[i - 1] = math.sqrt(num / den)
    jm = np.diag(diag) + np.diag(off, 1) + np.diag(off, -1)
    x = np.sort(np.linalg.eigvalsh(jm))
    # Newton polishing on the classical polynomial
    for _ in range(4):
        p, dp = _jacobi_p_std(x, a, b, q)
        x = x - p / dp
    _, dp = _jacobi_p_std(x, a, b, q)
    c = (2.0 ** (a + b + 1.0) * math.gamma(a + q + 1.0) * math.gamma(b + q + 1.0)
         / (math.gamma(q + 1.0) * math.gamma(a + b + q + 1.0)))
    w = c / ((1.0 - x * x) * dp * dp)
    del k
    return x, w


def gauss_lobatto_nodes(n: int) -> np.ndarray:
    """Legendre-Gauss-Lobatto nodes (n+1 points) on [-1, 1], ascending."""
    if n == 1:
        return np.array([-1.0, 1.0])
    xi, _ = gauss_jacobi(n - 1, 1.0, 1.0)
    return np.concatenate(([-1.0], xi, [1.0]))


def vandermonde_1d(n: int, r) -> np.ndarray:
    """Orthonormal Legendre Vandermonde V[i, j] = P_j(r_i), j = 0..n."""
    r = np.asarray(r, dtype=np.float64)
    return np.stack([jacobi_p(r, 0.0, 0.0, j) for j in range(n + 1)], axis=1)


def grad_vandermonde_1d(n: int, r) -> np.ndarray:
    r = np.asarray(r, dtype=np.float64)
    return np.stack([grad_jacobi_p(r, 0.0, 0.0, j) for j in range(n + 1)], axis=1)


# ---------------------------------------------------------------------------
# Simplex bases (orthonormal PKD) and their gradients
# ---------------------------------------------------------------------------

def _pow(base: np.ndarray, e: int) -> np.ndarray:
    """base**e with the convention that a negative exponent gives 0.

    Negative exponents only arise multiplied by a factor that vanishes for
    that mode (a derivative of a constant), so 0 is the correct value.
    """
    if e < 0:
        return np.zeros_like(base)
    return base ** e


def tri_rs_to_ab(r, s):
    r = np.asarray(r, dtype=np.float64)
    s = np.asarray(s, dtype=np.float64)
    a = np.where(np.abs(1.0 - s) > 1e-14, 2.0 * (1.0 + r) / np.where(np.abs(1.0 - s) > 1e-14, 1.0 - s, 1.0) - 1.0, -1.0)
    return a, s


def tri_modes(n: int):
    return [(i, j) for i in range(n + 1) for j in range(n + 1 - i)]


def tri_basis(n: int, r, s):
    """Orthonormal triangle basis and its r, s derivatives at (r, s).

    psi_ij = sqrt(2) P_i(a) (1-b)^i P_j^{(2i+1,0)}(b) on the reference
    triangle {r, s >= -1, r + s <= 0} with collapsed coordinates
    a = 2(1+r)/(1-s) - 1, b = s.  Mode order (i outer, j inner) follows
    the warped product's modal index in tensor_simplex.jl:92-95.
    """
    a, b = tri_rs_to_ab(r, s)
    modes = tri_modes(n)
    V = np.empty((a.size, len(modes)))
    Vr = np.empty_like(V)
    Vs = np.empty_like(V)
    sq2 = math.sqrt(2.0)
    for col, (i, j) in enumerate(modes):
        f = jacobi_p(a, 0, 0, i)
        df = grad_jacobi_p(a, 0, 0, i)
        g = jacobi_p(b, 2 * i + 1, 0, j)
        dg = grad_jacobi_p(b, 2 * i + 1, 0, j)
        omb = 1.0 - b
        V[:, col] = sq2 * f * _pow(omb, i) * g
        # d/dr: da/dr = 2/(1-b)
        Vr[:, col] = sq2 * 2.0 * df * _pow(omb, i - 1) * g
        # d/ds: da/ds = (1+a)/(1-b), db/ds = 1
        Vs[:, col] = sq2 * (df * (1.0 + a) * _pow(omb, i - 1) * g
                            + f * (-i * _pow(omb, i - 1) * g + _pow(omb, i) * dg))
    return V, Vr, Vs


def tet_rst_to_abc(r, s, t):
    r = np.asarray(r, dtype=np.float64)
    s = np.asarray(s, dtype=np.float64)
    t = np.asarray(t, dtype=np.float64)
    den_a = -s - t
    ok_a = np.abs(den_a) > 1e-14
    a = np.where(ok_a, 2.0 * (1.0 + r) / np.where(ok_a, den_a, 1.0) - 1.0, -1.0)
    den_b = 1.0 - t
    ok_b = np.abs(den_b) > 1e-14
    b = np.where(ok_b, 2.0 * (1.0 + s) / np.where(ok_b, den_b, 1.0) - 1.0, -1.0)
    return a, b, t


def tet_modes(n: int):
    return [(i, j, k) for i in range(n + 1) for j in range(n + 1 - i)
            for k in range(n + 1 - i - j)]


def tet_basis(n: int, r, s, t):
    """Orthonormal tetrahedron basis and its r, s, t derivatives.

    psi_ijk = 2 sqrt(2) P_i(a) (1-b)^i P_j^{(2i+1,0)}(b) (1-c)^{i+j}
    P_k^{(2i+2j+2,0)}(c) with a = 2(1+r)/(-s-t) - 1, b = 2(1+s)/(1-t) - 1,
    c = t.  Derivatives by the chain rule with
    da/dr = 4/((1-b)(1-c)), da/ds = da/dt = 2(1+a)/((1-b)(1-c)),
    db/ds = 2/(1-c), db/dt = (1+b)/(1-c).
    """
    a, b, c = tet_rst_to_abc(r, s, t)
    modes = tet_modes(n)
    V = np.empty((a.size, len(modes)))
    Vr = np.empty_like(V)
    Vs = np.empty_like(V)
    Vt = np.empty_like(V)
    k0 = 2.0 * math.sqrt(2.0)
    omb = 1.0 - b
    omc = 1.0 - c
    for col, (i, j, k) in enumerate(modes):
        f = jacobi_p(a, 0, 0, i)
        df = grad_jacobi_p(a, 0, 0, i)
        pj = jacobi_p(b, 2 * i + 1, 0, j)
        dpj = grad_jacobi_p(b, 2 * i + 1, 0, j)
        pk = jacobi_p(c, 2 * i + 2 * j + 2, 0, k)
        dpk = grad_jacobi_p(c, 2 * i + 2 * j + 2, 0, k)
        g = _pow(omb, i) * pj
        dg = -i * _pow(omb, i - 1) * pj + _pow(omb, i) * dpj
        h = _pow(omc, i + j) * pk
        dh = -(i + j) * _pow(omc, i + j - 1) * pk + _pow(omc, i + j) * dpk
        hm1 = _pow(omc, i + j - 1) * pk          # h / (1 - c)
        gm1 = _pow(omb, i - 1) * pj              # g / (1 - b)
        V[:, col] = k0 * f * g * h
        Vr[:, col] = k0 * 4.0 * df * gm1 * hm1
        term_a = k0 * 2.0 * (1.0 + a) * df * gm1 * hm1
        Vs[:, col] = term_a + k0 * f * dg * 2.0 * hm1
        Vt[:, col] = term_a + k0 * f * dg * (1.0 + b) * hm1 + k0 * f * g * dh
    return V, Vr, Vs, Vt


# ---------------------------------------------------------------------------
# Interpolation nodes on simplices
# ---------------------------------------------------------------------------

def _warp_factor(n: int, rout: np.ndarray) -> np.ndarray:
    """1-D warp from equispaced to LGL nodes, blended to vanish at +-1."""
    lgl = gauss_lobatto_nodes(n)
    req = np.linspace(-1.0, 1.0, n + 1)
    veq = vandermonde_1d(n, req)
    pmat = vandermonde_1d(n, rout).T                   # (n+1, Nr)
    lmat = np.linalg.solve(veq.T, pmat)               # Lagrange basis at rout
    warp = lmat.T @ (lgl - req)
    zerof = (np.abs(rout) < 1.0 - 1.0e-10).astype(np.float64)
    sf = 1.0 - (zerof * rout) ** 2
    return warp / np.where(sf != 0.0, sf, 1.0) + warp * (zerof - 1.0)


def tri_nodes(n: int, alpha: float = 0.0):
    """Warp-and-blend interpolation nodes of degree ``n`` on the triangle.

    ``alpha`` is the interior blending exponent of Warburton's construction.
    The mapping nodes of the reference's ``RefElemData`` use alpha = 0: with
    it the reference's degree-4 curved-triangle golden (test/runtests.jl:57)
    is reproduced to 2e-15, and not with the optimised alpha(4) = 0.1001 of
    Hesthaven & Warburton's table; degrees <= 3 do not depend on alpha.
    Ordering: the equispaced loop (L1 outer, L3 inner), which for n = 1
    gives the vertices (-1,-1), (1,-1), (-1,1).
    """
    if n == 0:
        return np.array([-1.0 / 3.0]), np.array([-1.0 / 3.0])
    l1, l3 = [], []
    for i in range(n + 1):
        for j in range(n + 1 - i):
            l1.append(i / n)
            l3.append(j / n)
    l1 = np.array(l1)
    l3 = np.array(l3)
    l2 = 1.0 - l1 - l3
    x = -l2 + l3
    y = (-l2 - l3 + 2.0 * l1) / math.sqrt(3.0)
    blend1 = 4.0 * l2 * l3
    blend2 = 4.0 * l1 * l3
    blend3 = 4.0 * l1 * l2
    warpf1 = _warp_factor(n, l3 - l2)
    warpf2 = _warp_factor(n, l1 - l3)
    warpf3 = _warp_factor(n, l2 - l1)
    warp1 = blend1 * warpf1 * (1.0 + (alpha * l1) ** 2)
    warp2 = blend2 * warpf2 * (1.0 + (alpha * l2) ** 2)
    warp3 = blend3 * warpf3 * (1.0 + (alpha * l3) ** 2)
    x = x + warp1 + math.cos(2.0 * math.pi / 3.0) * warp2 + math.cos(4.0 * math.pi / 3.0) * warp3
    y = y + math.sin(2.0 * math.pi / 3.0) * warp2 + math.sin(4.0 * math.pi / 3.0) * warp3
    # equilateral (x, y) -> reference (r, s)
    b1 = (math.sqrt(3.0) * y + 1.0) / 3.0
    b2 = (-3.0 * x - math.sqrt(3.0) * y + 2.0) / 6.0
    b3 = (3.0 * x - math.sqrt(3.0) * y + 2.0) / 6.0
    r = -b2 + b3 - b1
    s = -b2 - b3 + b1
    return r, s


def _face_warp(n: int, l1, l2, l3):
    """Warp-and-blend shift (dx, dy) of points of an equilateral triangle
    with barycentric coordinates l1, l2, l3 (alpha = 0): the 1-D warp of the
    edge opposite each vertex blended by the product of the other two
    coordinates -- the triangle construction of tri_nodes, in the form
    Warburton (2006) uses on the faces of the tetrahedron."""
    w1 = 4.0 * l2 * l3 * _warp_factor(n, l3 - l2)
    w2 = 4.0 * l1 * l3 * _warp_factor(n, l1 - l3)
    w3 = 4.0 * l1 * l2 * _warp_factor(n, l2 - l1)
    dx = w1 + math.cos(2.0 * math.pi / 3.0) * w2 + math.cos(4.0 * math.pi / 3.0) * w3
    dy = math.sin(2.0 * math.pi / 3.0) * w2 + math.sin(4.0 * math.pi / 3.0) * w3
    return dx, dy


def _tet_equispaced(n: int):
    r, s, t = [], [], []
    for k in range(n + 1):
        for j in range(n + 1 - k):
            for i in range(n + 1 - k - j):
                r.append(-1.0 + 2.0 * i / n)
                s.append(-1.0 + 2.0 * j / n)
                t.append(-1.0 + 2.0 * k / n)
    return np.array(r), np.array(s), np.array(t)


def tet_nodes(n: int, kind: str = "warp_blend"):
    """Degree-``n`` interpolation nodes on the tetrahedron.

    ``kind="warp_blend"`` (default): Warburton's warp-and-blend nodes (T.
    Warburton, J. Eng. Math. 56 (2006) 247-262), the tetrahedral counterpart
    of tri_nodes with the same blending exponent alpha = 0: the equispaced
    lattice in an equilateral tetrahedron is shifted, face by face, by the
    triangle's warp in the face's tangent plane, blended into the volume by
    Lb Lc Ld / ((Lb + La/2)(Lc + La/2)(Ld + La/2)) for the face La = 0; on
    the faces the nodes are exactly the triangle's, on the edges the
    Gauss-Lobatto points.  ``kind="equispaced"``: the plain lattice.
    Ordering (both): the lattice index of t outermost, r innermost; for n =
    1 the vertices (-1,-1,-1), (1,-1,-1), (-1,1,-1), (-1,-1,1).  These are
    the mapping nodes of the curved tetrahedra (``nodes(Tet(), N)`` of the
    reference's RefElemData, ref_elem_data.jl:77).
    """
    r, s, t = _tet_equispaced(n)
    if kind == "equispaced" or n <= 2:
        # degrees <= 2: the Gauss-Lobatto points are equispaced
        return r, s, t
    if kind != "warp_blend":
        raise ValueError(kind)
    L1, L2 = (1.0 + t) / 2.0, (1.0 + s) / 2.0
    L3, L4 = -(1.0 + r + s + t) / 2.0, (1.0 + r) / 2.0
    v1 = np.array([-1.0, -1.0 / math.sqrt(3.0), -1.0 / math.sqrt(6.0)])
    v2 = np.array([1.0, -1.0 / math.sqrt(3.0), -1.0 / math.sqrt(6.0)])
    v3 = np.array([0.0, 2.0 / math.sqrt(3.0), -1.0 / math.sqrt(6.0)])
    v4 = np.array([0.0, 0.0, 3.0 / math.sqrt(6.0)])
    # orthonormal tangents of the four faces
    t1 = [v2 - v1, v2 - v1, v3 - v2, v3 - v1]
    t2 = [v3 - 0.5 * (v1 + v2), v4 - 0.5 * (v1 + v2), v4 - 0.5 * (v2 + v3), v4 - 0.5 * (v1 + v3)]
    t1 = [x / np.linalg.norm(x) for x in t1]
    t2 = [x / np.linalg.norm(x) for x in t2]
    xyz = np.outer(L3, v1) + np.outer(L4, v2) + np.outer(L2, v3) + np.outer(L1, v4)
    shift = np.zeros_like(xyz)
    tol = 1.0e-10
    faces = [(L1, L2, L3, L4), (L2, L1, L3, L4), (L3, L1, L4, L2), (L4, L1, L3, L2)]
    for f, (La, Lb, Lc, Ld) in enumerate(faces):
        w1, w2 = _face_warp(n, Lb, Lc, Ld)
        blend = Lb * Lc * Ld
        denom = (Lb + 0.5 * La) * (Lc + 0.5 * La) * (Ld + 0.5 * La)
        blend = np.where(denom > tol, blend / np.where(denom > tol, denom, 1.0), blend)
        shift += np.outer(blend * w1, t1[f]) + np.outer(blend * w2, t2[f])
        # nodes of this face that lie on an edge take the face's warp alone
        on_edge = (La < tol) & (((Lb > tol).astype(int) + (Lc > tol) + (Ld > tol)) < 3)
        shift[on_edge] = np.outer(w1[on_edge], t1[f]) + np.outer(w2[on_edge], t2[f])
    xyz = xyz + shift
    # equilateral -> reference coordinates: xyz = v1 + (r+1)/2 (v2-v1) + (s+1)/2 (v3-v1) + (t+1)/2 (v4-v1)
    A = 0.5 * np.column_stack([v2 - v1, v3 - v1, v4 - v1])
    rhs = xyz - 0.5 * (v2 + v3 + v4 - v1)
    rst = np.linalg.solve(A, rhs.T)
    return rst[0], rst[1], rst[2]
