"""Mesh connectivity and geometric factors on curved periodic meshes."""
import numpy as np
import pytest


def _sd(pkg, shape, p, cells, metrics, warp=0.1):
    R, M = pkg.reference, pkg.mesh
    ra = R.reference_approximation("ModalTensor", shape, p, mapping_degree=p)
    d = 2 if shape == "Tri" else 3
    lim = ((0.0, 1.0),) * d
    mesh = M.uniform_periodic_mesh(ra, lim, (cells,) * d)
    if warp:
        mesh = M.warp_mesh(mesh, ra, "Chan", warp, (1.0,) * d)
    return M.spatial_discretization(mesh, ra, metrics=metrics)


@pytest.mark.parametrize("shape,p,cells", [("Tri", 4, 4), ("Tet", 3, 2), ("Tet", 4, 3)])
@pytest.mark.parametrize("metrics", ["Exact", "ChanWilcox"])
def test_watertight_and_conforming(pkg, shape, p, cells, metrics):
    sd = _sd(pkg, shape, p, cells, metrics, warp=0.05)
    assert pkg.mesh.check_facet_nodes(sd) < 1e-12
    assert pkg.mesh.check_normals(sd) < 1e-10
    mapP = sd.mesh.mapP.reshape(-1) - 1
    assert np.array_equal(mapP[mapP], np.arange(mapP.size))      # involution
    assert np.all(mapP != np.arange(mapP.size))                   # no self-match
    assert sd.geometric_factors.J_q.min() > 0


@pytest.mark.parametrize("shape", ["Tri", "Tet"])
def test_mesh_volume(pkg, shape):
    sd = _sd(pkg, shape, 3, 2, "Exact", warp=0.05)
    vol = (sd.reference_approximation.W[None, :] * sd.geometric_factors.J_q).sum()
    assert abs(vol - 1.0) < 1e-10


def test_uniform_element_counts(pkg):
    R, M = pkg.reference, pkg.mesh
    ra = R.reference_approximation("ModalTensor", "Tri", 2, mapping_degree=1)
    assert M.uniform_periodic_mesh(ra, ((0, 1), (0, 1)), (16, 16)).N_e == 512
    ra = R.reference_approximation("ModalTensor", "Tet", 2, mapping_degree=1)
    assert M.uniform_periodic_mesh(ra, ((0, 1),) * 3, (4, 4, 4)).N_e == 384
