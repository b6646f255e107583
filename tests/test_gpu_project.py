"""L2 projection of initial data on the GPU (sse_project_function) against
the host restatement of project_function (Solvers.jl:396-418)."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["vortex_tri_modal", "tgv_tet_modal", "tgv_tet_p5", "tgv_tet_p6",
                                  "multi_tri", "multi_tet"])
def test_projection_matches_host(name, gpu_lib, pkg):
    host, _ = cases.make(name)
    sd = host.sd
    if "tet" in name:
        ic = pkg.solver.TaylorGreenVortex(1.4, 0.1)
    else:
        ic = pkg.setups.vortex_tri(cells=2, p=2).initial_data
    want = pkg.solver.initialize(ic, sd)
    got = pkg.solver.initialize(ic, sd, projection="gpu")
    err = np.abs(got - want).max() / np.abs(want).max()
    assert err < 1e-12, err


def test_projection_device_buffers(gpu_lib, pkg):
    import torch
    host, _ = cases.make("tgv_tet_modal")
    sd = host.sd
    ra = sd.reference_approximation
    uq = pkg.solver.TaylorGreenVortex(1.4, 0.1).evaluate(sd.mesh.xyzq, 0.0).transpose(0, 2, 1)
    uq = np.ascontiguousarray(uq)
    a = pkg.gb300.project_function(ra, sd.geometric_factors.J_q, uq)
    b = pkg.gb300.project_function(ra, torch.from_numpy(sd.geometric_factors.J_q).cuda(),
                                   torch.from_numpy(uq).cuda())
    assert np.array_equal(a, b.cpu().numpy())


def test_projection_rejects_a_negative_jacobian(gpu_lib, pkg):
    """A mass matrix that is not positive definite is an error, as the
    reference's cholesky throws."""
    host, _ = cases.make("vortex_tri_modal")
    sd = host.sd
    J = sd.geometric_factors.J_q.copy()
    J[3] *= -1.0
    uq = np.ones((sd.N_e, 4, J.shape[1]))
    with pytest.raises(pkg.SSEError) as e:
        pkg.gb300.project_function(sd.reference_approximation, J, uq)
    assert e.value.code == pkg.abi.SSE_ERR_NONPHYSICAL
