"""Geometric factors on the GPU (sse_geometric_factors) against the host
FP64 restatement of GeometricFactors (mesh.jl:229-282, 284-339, 410-506)
and project_jacobian! (SpatialDiscretizations.jl:310-317), field by field,
and through the residual they feed."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu

M, R = cases.M, cases.R

# (approximation, element, degree, cells, metrics, project_jacobian)
CASES = [
    ("ModalTensor", "Tri", 4, 8, "Exact", True),
    ("NodalTensor", "Tri", 3, 6, "Exact", True),
    ("ModalTensor", "Tri", 4, 8, "ChanWilcox", False),
    ("ModalTensor", "Tri", 2, 5, "Exact", False),
    ("ModalTensor", "Tet", 2, 3, "Exact", False),
    ("ModalTensor", "Tet", 3, 3, "Exact", True),
    ("ModalTensor", "Tet", 4, 3, "ChanWilcox", False),
    ("NodalTensor", "Tet", 3, 2, "ChanWilcox", False),
    ("ModalTensor", "Tet", 5, 2, "ChanWilcox", False),
    ("ModalTensor", "Tet", 6, 2, "ChanWilcox", False),
]

FIELDS = ("J_q", "Lambda_q", "J_f", "nJf", "nJq")


def _mesh(approx, shape, p, cells):
    ra = R.reference_approximation(approx, shape, p, mapping_degree=p)
    d = 2 if shape == "Tri" else 3
    L = 2 * np.pi
    mesh = M.uniform_periodic_mesh(ra, ((0.0, L),) * d, (cells,) * d)
    return ra, M.warp_mesh(mesh, ra, "Chan", 0.1 if d == 2 else 0.05, (L,) * d)


def _host(mesh, ra, metrics, project):
    sd = M.spatial_discretization(mesh, ra, metrics=metrics, project_jac=project)
    return sd.geometric_factors


@pytest.mark.parametrize("approx,shape,p,cells,metrics,project", CASES)
def test_fields_match_host(approx, shape, p, cells, metrics, project, gpu_lib, pkg):
    ra, mesh = _mesh(approx, shape, p, cells)
    want = _host(mesh, ra, metrics, project)
    got = pkg.gb300.geometric_factors(mesh, ra, metrics, project)
    for f in FIELDS:
        a, b = getattr(got, f), getattr(want, f)
        assert a.shape == b.shape, f
        scale = np.abs(b).max()
        err = np.abs(a - b).max() / scale
        # FP64 with another summation order (and FMA) than numpy's BLAS
        assert err <= 2e-13, (f, err)


def test_device_buffers_match_host_buffers(gpu_lib, pkg):
    import torch
    ra, mesh = _mesh("ModalTensor", "Tet", 4, 3)
    got = pkg.gb300.geometric_factors(mesh, ra, "ChanWilcox", False)
    xyz = [torch.from_numpy(x).cuda() for x in mesh.xyz]
    dev = pkg.gb300.geometric_factors(mesh, ra, "ChanWilcox", False, xyz=xyz)
    for f in FIELDS:
        t = getattr(dev, f)
        assert t.is_cuda
        assert np.array_equal(t.cpu().numpy(), getattr(got, f)), f


def test_free_stream_and_normals(gpu_lib, pkg):
    """Metric identities of the reference's checks (SpatialDiscretizations.jl:
    425-430 normals, free-stream preservation of the curl metrics) on the
    GPU-built factors: neighbours' facet normals cancel, and a constant state
    has a round-off residual."""
    host, _ = cases.make("tgv_tet_modal")
    sd = host.sd
    sd2 = M.spatial_discretization(sd.mesh, sd.reference_approximation, metrics=sd.metrics,
                                   geometry="gpu")
    # the host-built factors' bound (tests/test_mesh_geometry.py), and no
    # worse than the host's own mismatch
    assert M.check_normals(sd2) < 1e-10
    assert M.check_normals(sd2) <= 2 * M.check_normals(sd) + 1e-12
    h2 = pkg.solver.HostArrays(host.law, sd2, host.form)
    uc = pkg.solver.initialize(pkg.solver.EulerPeriodicTest(3, strength=0.0), sd2)
    r = pkg.GB300Solver(h2).residual(uc)
    assert np.abs(r).max() < 1e-10 * np.abs(uc).max()


@pytest.mark.parametrize("name", ["vortex_tri_modal", "tgv_tet_modal", "adv_tri_modal", "adv_tet_modal"])
def test_residual_with_gpu_geometry(name, gpu_lib, pkg):
    host, u = cases.make(name)
    sd = host.sd
    sd2 = M.spatial_discretization(sd.mesh, sd.reference_approximation, metrics=sd.metrics,
                                   geometry="gpu")
    h2 = pkg.solver.HostArrays(host.law, sd2, host.form)
    r1 = pkg.GB300Solver(host).residual(u)
    r2 = pkg.GB300Solver(h2).residual(u)
    err = np.linalg.norm(r1 - r2) / np.linalg.norm(r1)
    assert err < 1e-11, err
