"""Meshes whose element count is not a multiple of the elements per block:
50 triangles leave the last block of flux differencing (eight 16-thread
teams per block; four 32-thread teams in the mixed form's FP32 phase B) with
two live teams, and 18 triangles the last block of StandardForm (four
32-thread teams per block) with two of four.  The idle teams of the last
block run on a valid element's data for the block's barriers and must leave
every output untouched: residual, nodal states, mixed form, vector-Jacobian
product and a few Runge-Kutta steps against the oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.oracle import Oracle, rel2, roundoff_floor

pytestmark = pytest.mark.gpu


def _problem(pkg, form):
    s = pkg.setups
    # a weak vortex on 5 x 5 cells: resolved enough to stay physical
    pb = s.vortex_tri(cells=5, p=3, strength=1.0) if form == "fd" else s.advection_tri(cells=3, p=4)
    host = pb.host_arrays()
    assert host.N_e == (50 if form == "fd" else 18)
    return pb, host, s.perturbed(pb.u0, 7, 1.0e-3)


@pytest.mark.parametrize("form", ["fd", "std"])
def test_residual_and_steps_on_partial_blocks(gpu_lib, pkg, form):
    pb, host, u = _problem(pkg, form)
    gpu = pkg.GB300Solver(host)
    o = Oracle(host)
    got = gpu.residual(u)
    want = o.residual(u)
    assert rel2(got, want) <= max(1e-12, 4.0 * roundoff_floor(host, u))
    uq_g, uf_g = gpu.nodal_values(u)
    uq_o, uf_o = o.nodal_values(u)
    assert rel2(uq_g, uq_o) <= 1e-12 and rel2(uf_g, uf_o) <= 1e-12
    scheme = 0 if form == "fd" else 1
    ug = u.copy()
    gpu.rk_steps(ug, 3, 1e-3, scheme)
    assert rel2(ug, o.rk_steps(u, 3, 1e-3, scheme)) <= 1e-12


@pytest.mark.parametrize("form", ["fd", "std"])
def test_vjp_on_partial_blocks(gpu_lib, pkg, form):
    _, host, u = _problem(pkg, form)
    G = pkg.GB300Solver(host)
    rng = np.random.default_rng(5)
    lam = rng.standard_normal(u.shape)
    v = rng.standard_normal(u.shape)
    mu = G.residual_vjp(u, lam)
    _, jv = O.TangentOracle(host).jvp(u, v)
    lhs, rhs = float(np.vdot(lam, jv)), float(np.vdot(mu, v))
    scale = max(float(np.sum(np.abs(lam * jv))), float(np.sum(np.abs(mu * v))))
    assert abs(lhs - rhs) / scale < 1e-11


def test_mixed_form_on_partial_blocks(gpu_lib, pkg):
    _, host, u = _problem(pkg, "fd")
    a = pkg.GB300Solver(host)
    b = pkg.GB300Solver(host)
    b.set_precision(pkg.abi.SSE_MIXED)
    ua, ub = u.copy(), u.copy()
    a.rk_steps(ua, 5, 1e-3, 0)
    b.rk_steps(ub, 5, 1e-3, 0)
    assert rel2(ub, ua) < 1e-6
