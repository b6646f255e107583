"""The CPU oracle against the reference's own invariants (its tests assert
conservation and entropy/energy conservation to 1e-10, test/runtests.jl:
57-59, 120, 127-128): discrete conservation, free-stream preservation and
round-off entropy conservation of the EC scheme on curved meshes."""
import numpy as np
import pytest

import cases
from oracle.oracle import Oracle


@pytest.mark.parametrize("name", cases.NAMES + cases.MULTI_NAMES)
def test_conservation(name):
    host, u = cases.make(name)
    o = Oracle(host)
    du = o.residual(u)
    cons = o.conservation_residual(u, du)[: host.N_c]
    scale = np.abs(du).max() * np.abs(host.WJ).sum()
    assert np.abs(cons).max() < 1e-12 * scale


@pytest.mark.parametrize("name", ["vortex_tri_ec", "tgv_tet_ec", "multi_tri_ec", "multi_tet_ec",
                                  "vortex_tri_chandra_ec", "tgv_tet_chandra_ec"])
def test_entropy_conservation(name):
    host, u = cases.make(name)
    o = Oracle(host)
    du = o.residual(u)
    s = o.conservation_residual(u, du)[host.N_c]
    scale = np.abs(du).max() * np.abs(host.WJ).sum() * 10
    assert abs(s) < 1e-12 * scale


@pytest.mark.parametrize("name", ["vortex_tri_modal", "tgv_tet_modal", "tgv_tet_nodal", "multi_tri",
                                  "multi_tri_nodal", "multi_tet", "vortex_tri_chandra", "tgv_tet_chandra"])
def test_free_stream_preservation(name):
    host, _ = cases.make(name)
    S = cases.S
    d = host.cfg.d

    class Const:
        N_c = d + 2

        def evaluate(self, x, t=0.0):
            one = np.ones_like(x[0])
            cols = [1.2 * one] + [(0.3 - 0.2 * m) * one for m in range(d)] + [2.5 * one]
            return np.stack(cols, -1)
    u = S.initialize(Const(), host.sd)
    du = Oracle(host).residual(u)
    assert np.abs(du).max() < 1e-11


def _energy_rate_wa(host, u, du):
    """sum_k u' M dudt with the weight-adjusted mass matrix
    M = inv(V' diag(W/J) V) (EnergyConservationAnalysis, conservation.jl:161-175)."""
    V = host.sd.reference_approximation.V
    total = 0.0
    for k in range(host.N_e):
        Minv = V.T @ (host.JinvW[k][:, None] * V)
        total += u[k, 0] @ np.linalg.solve(Minv, du[k, 0])
    return total


def test_energy_rate_lax_friedrichs_and_central():
    host, u = cases.make("adv_tri_modal")
    du = Oracle(host).residual(u)
    assert _energy_rate_wa(host, u, du) < 0.0
    host, u = cases.make("adv_tri_central")
    du = Oracle(host).residual(u)
    assert abs(_energy_rate_wa(host, u, du)) < 1e-12 * np.abs(du).max()
