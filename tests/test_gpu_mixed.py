"""The mixed FP32/FP64 form (sse_set_precision(SSE_MIXED)) against the FP64
form on the same handle and inputs.

Bounds: the solution state after CarpenterKennedy2N54 steps agrees with the
FP64 trajectory to <= 1e-6 relative (2-norm), the accuracy the mixed form
is specified at; the residual itself agrees to <= 1e-4 relative; discrete
conservation (computed in FP64 from the mixed residual) holds to FP32
round-off of the fluxes.
"""
import numpy as np
import pytest

import cases
from oracle.oracle import rel2

pytestmark = pytest.mark.gpu


def _pair(pkg, name):
    host, u = cases.make(name)
    fp64 = pkg.GB300Solver(host)
    mixed = pkg.GB300Solver(host)
    mixed.set_precision(pkg.abi.SSE_MIXED)
    return host, u, fp64, mixed


@pytest.mark.parametrize("name", ["vortex_tri_modal", "vortex_tri_nodal", "tgv_tet_modal",
                                  "tgv_tet_ec", "tgv_tet_p5", "tgv_tet_p2", "multi_tri",
                                  "multi_tri_nodal", "multi_tet"])
def test_mixed_residual_close_to_fp64(gpu_lib, pkg, name):
    host, u, fp64, mixed = _pair(pkg, name)
    want = fp64.residual(u)
    got = mixed.residual(u)
    err = rel2(got, want)
    print(f"{name}: mixed residual rel2 vs FP64 {err:.2e}")
    assert err <= 1e-4


@pytest.mark.parametrize("name,steps,dt", [("vortex_tri_modal", 20, 2e-3), ("tgv_tet_modal", 20, 1e-3),
                                           ("multi_tet", 20, 1e-3)])
def test_mixed_trajectory_within_1e6(gpu_lib, pkg, name, steps, dt):
    host, u, fp64, mixed = _pair(pkg, name)
    a = u.copy()
    b = u.copy()
    fp64.rk_steps(a, steps, dt)
    mixed.rk_steps(b, steps, dt)
    err = rel2(b, a)
    print(f"{name}: state rel2 after {steps} CK2N54 steps {err:.2e}")
    assert err <= 1e-6


@pytest.mark.parametrize("name", ["vortex_tri_ec", "tgv_tet_ec", "multi_tet_ec"])
def test_mixed_conservation_and_entropy(gpu_lib, pkg, name):
    host, u, fp64, mixed = _pair(pkg, name)
    du = mixed.residual(u)
    out = fp64.conservation_residual(u, du)
    scale = np.abs(du).max() * np.abs(host.WJ).sum()
    print(f"{name}: mixed conservation {out[:host.N_c] / scale}, entropy {out[host.N_c] / scale}")
    assert np.abs(out[: host.N_c]).max() <= 1e-6 * scale
    assert abs(out[host.N_c]) <= 1e-5 * scale


@pytest.mark.parametrize("name", ["adv_tri_modal", "vortex_tri_chandra"])
def test_mixed_rejected_outside_flux_differencing_euler(gpu_lib, pkg, name):
    host, _ = cases.make(name)
    gpu = pkg.GB300Solver(host)
    with pytest.raises(pkg.SSEError) as ei:
        gpu.set_precision(pkg.abi.SSE_MIXED)
    assert ei.value.code == pkg.abi.SSE_ERR_UNSUPPORTED
