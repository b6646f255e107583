"""Reference-element operators: the properties the reference itself checks
(SpatialDiscretizations.jl:425-470) and exactness of the 1-D building blocks."""
import numpy as np
import pytest


@pytest.mark.parametrize("shape", ["Tri", "Tet"])
@pytest.mark.parametrize("approx", ["ModalTensor", "NodalTensor"])
@pytest.mark.parametrize("p", [2, 4, 5])
def test_sbp_property(pkg, shape, approx, p):
    ra = pkg.reference.reference_approximation(approx, shape, p, mapping_degree=p)
    assert max(pkg.reference.check_sbp_property(ra)) < 1e-13


@pytest.mark.parametrize("shape", ["Tri", "Tet"])
@pytest.mark.parametrize("p", [3, 4, 5])
def test_modal_basis_orthonormal_and_facet_map(pkg, shape, p):
    R = pkg.reference
    P = pkg.polynomials
    ra = R.reference_approximation("ModalTensor", shape, p, mapping_degree=p)
    V = ra.V
    assert np.abs(V.T @ np.diag(ra.W) @ V - np.eye(ra.N_p)).max() < 1e-13
    re = ra.reference_element
    basis = P.tri_basis if shape == "Tri" else P.tet_basis
    assert np.abs(V - basis(p, *re.rstq)[0]).max() < 1e-12
    assert np.abs(ra.R @ V - basis(p, *re.rstf)[0]).max() < 1e-12
    # warped factors reproduce the dense Vandermonde
    assert np.abs(ra.warped.dense() - V).max() == 0.0


@pytest.mark.parametrize("ab", [(0, 0), (1, 0), (2, 0)])
def test_gauss_jacobi_exactness(pkg, ab):
    a, b = ab
    x, w = pkg.polynomials.gauss_jacobi(6, a, b)
    # int_{-1}^{1} x^k (1-x)^a (1+x)^b exact for k <= 11, via the 40-point rule
    X, Wt = np.polynomial.legendre.leggauss(40)
    for k in range(12):
        ref = np.sum(Wt * X ** k * (1 - X) ** a * (1 + X) ** b)
        assert abs(np.sum(w * x ** k) - ref) < 1e-13


@pytest.mark.parametrize("n", [1, 3, 4, 6])
def test_simplex_derivative_matrices_exact(pkg, n):
    P = pkg.polynomials
    r, s = P.tri_nodes(n)
    V, Vr, Vs = P.tri_basis(n, r, s)
    Dr = np.linalg.solve(V.T, Vr.T).T
    Ds = np.linalg.solve(V.T, Vs.T).T
    f = r ** n + r * s ** (n - 1) + 2.0
    assert np.abs(Dr @ f - (n * r ** (n - 1) + s ** (n - 1))).max() < 1e-12
    assert np.abs(Ds @ f - ((n - 1) * r * s ** max(n - 2, 0) if n > 1 else 0 * s)).max() < 1e-12
    r, s, t = P.tet_nodes(n)
    V, Vr, Vs, Vt = P.tet_basis(n, r, s, t)
    Dt = np.linalg.solve(V.T, Vt.T).T
    c = 1.0 if n >= 2 else 0.0            # r t is degree 2
    g = t ** n + c * r * t + s
    assert np.abs(Dt @ g - (n * t ** (n - 1) + c * r)).max() < 1e-11


def test_warp_and_blend_vertices_and_edges(pkg):
    P = pkg.polynomials
    r, s = P.tri_nodes(1)
    assert np.allclose(np.stack([r, s], 1), [[-1, -1], [1, -1], [-1, 1]])
    r, s = P.tri_nodes(4)
    edge = np.sort(r[np.abs(s + 1) < 1e-14])
    assert np.abs(edge - P.gauss_lobatto_nodes(4)).max() < 1e-14


def _sorted_barycentric(points):
    """Each point's barycentric coordinates, sorted, as a sorted array (a
    set invariant under the simplex's symmetries)."""
    b = np.sort(np.round(np.asarray(points), 11) + 0.0, axis=1)
    return b[np.lexsort(b.T[::-1])]


@pytest.mark.parametrize("n", [3, 4, 5, 6])
def test_tet_warp_and_blend_faces_and_edges(pkg, n):
    """Every face of the tetrahedral set carries the triangle's warp-and-blend
    nodes and every edge the Gauss-Lobatto points; all nodes lie in the
    element, and n = 1 gives the vertices in the lattice order."""
    P = pkg.polynomials
    r, s, t = P.tet_nodes(n)
    lam = np.stack([(1 + t) / 2, (1 + s) / 2, -(1 + r + s + t) / 2, (1 + r) / 2], 1)
    assert lam.min() > -1e-13
    tr, ts = P.tri_nodes(n)
    tri = _sorted_barycentric(np.stack([(1 + ts) / 2, -(tr + ts) / 2, (1 + tr) / 2], 1))
    for f in range(4):
        on = np.abs(lam[:, f]) < 1e-12
        face = _sorted_barycentric(np.delete(lam[on], f, axis=1))
        assert face.shape == tri.shape and np.abs(face - tri).max() < 1e-12, f
    lgl = np.sort((1 + P.gauss_lobatto_nodes(n)) / 2)
    for a in range(4):
        for b in range(a + 1, 4):
            rest = [c for c in range(4) if c not in (a, b)]
            on = np.all(np.abs(lam[:, rest]) < 1e-12, axis=1)
            assert np.abs(np.sort(lam[on, a]) - lgl).max() < 1e-12, (a, b)
    r1, s1, t1 = P.tet_nodes(1)
    assert np.allclose(np.stack([r1, s1, t1], 1), [[-1, -1, -1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]])
    re, se, te = P.tet_nodes(n, "equispaced")
    assert np.allclose(np.sort(re), np.sort(-1 + 2 * np.round((re + 1) * n / 2) / n))
