"""The mixed FP32/FP64 form (sse_set_precision(SSE_MIXED)) against the FP64
form on the same handle and inputs.

Bounds: the solution state after CarpenterKennedy2N54 steps agrees with the
FP64 trajectory to <= 1e-6 relative (2-norm), the accuracy the mixed form
is specified at; the increment u(T) - u(0) agrees with the FP64 increment to
the residual's own accuracy (a short run moves the state little, so the
state error alone would hide the residual error); the residual itself
agrees to <= 1e-4 relative as a whole and per conserved variable; discrete
conservation (computed in FP64 from the mixed residual) holds to FP32
round-off of the fluxes.  Every check also runs on meshes built with the
reference's default exact metrics, which on curved tets do not preserve a
free stream (the FP64 residual of a constant state is O(1) there).
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


def component_errors(got, want):
    """rel2 of each conserved variable (component axis 1 of (N_e, N_c, N_p))."""
    return [rel2(got[:, c], want[:, c]) for c in range(want.shape[1])]


@pytest.mark.parametrize("name", ["vortex_tri_modal", "vortex_tri_nodal", "tgv_tet_modal",
                                  "tgv_tet_ec", "tgv_tet_p5", "tgv_tet_p2", "multi_tri",
                                  "multi_tri_nodal", "multi_tet"] + cases.EXACT_NAMES)
def test_mixed_residual_close_to_fp64(gpu_lib, pkg, name):
    host, u, fp64, mixed = _pair(pkg, name)
    want = fp64.residual(u)
    got = mixed.residual(u)
    err = rel2(got, want)
    comp = component_errors(got, want)
    print(f"{name}: mixed residual rel2 vs FP64 {err:.2e}, per variable "
          + " ".join(f"{c:.1e}" for c in comp))
    assert err <= 1e-4
    assert max(comp) <= 1e-4


@pytest.mark.parametrize("name", ["tgv_tet_exact", "tgv_tet_ec_exact", "tgv_tet_nodal_exact",
                                  "vortex_tri_exact", "tgv_tet_modal"])
def test_mixed_residual_of_a_constant_state(gpu_lib, pkg, name):
    """A constant state: the FP64 residual is the metric terms' free-stream
    error (O(1) on curved tets with exact metrics, round-off with the
    conservative-curl metrics); the mixed form must return the same, since
    its FP32 fluxes leave the reference pressure out and it adds that
    part back in FP64."""
    host, _, fp64, mixed = _pair(pkg, name)
    S = cases.S
    d = host.cfg.d

    class Const:
        N_c = d + 2

        def evaluate(self, x, t=0.0):
            one = np.ones_like(x[0])
            cols = [1.0 * one] + [0.0 * one] * d + [178.0 * one]
            return np.stack(cols, -1)
    u = S.initialize(Const(), host.sd)
    want = fp64.residual(u)
    got = mixed.residual(u)
    err = np.abs(got - want).max()
    print(f"{name}: constant state max|R64| {np.abs(want).max():.2e}, max|R_mixed - R64| {err:.2e}")
    assert err <= 1e-6 * max(np.abs(want).max(), 1.0)


@pytest.mark.parametrize("name,steps,dt", [("vortex_tri_modal", 20, 2e-3), ("tgv_tet_modal", 20, 1e-3),
                                           ("multi_tet", 20, 1e-3), ("vortex_tri_exact", 20, 2e-3),
                                           ("tgv_tet_exact", 20, 1e-3)])
def test_mixed_trajectory_within_1e6(gpu_lib, pkg, name, steps, dt):
    host, u, fp64, mixed = _pair(pkg, name)
    a = u.copy()
    b = u.copy()
    fp64.rk_steps(a, steps, dt)
    mixed.rk_steps(b, steps, dt)
    err = rel2(b, a)
    inc = rel2(b - u, a - u)
    comp = component_errors(b - u, a - u)
    print(f"{name}: after {steps} CK2N54 steps state rel2 {err:.2e}, increment rel2 {inc:.2e} "
          "(per variable " + " ".join(f"{c:.1e}" for c in comp) + ")")
    assert err <= 1e-6
    # the increment carries the residual's own error (bounded above at 1e-4)
    assert inc <= 1e-4


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
