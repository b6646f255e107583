"""The dual-number build of the oracle (oracle/sse_oracle_tangent.cpp), the
checker of the discrete adjoint: its value part is the oracle itself, bit for
bit, and its tangent part is the exact directional derivative -- checked
against central differences of the oracle and, for the linear advection
residual, against the residual of the direction itself."""
import numpy as np
import pytest

import cases
from oracle import oracle as O

# LF cases have kinks (max of wave speeds) where central differences lose
# accuracy for large steps; the smallest step error over a few steps is
# the measure of agreement
STEPS = (1e-5, 1e-6, 1e-7)


@pytest.fixture(scope="module", params=cases.NAMES)
def case(request):
    return cases.make(request.param)


def test_value_part_is_the_oracle(case):
    host, u = case
    rng = np.random.default_rng(3)
    v = rng.standard_normal(u.shape)
    r, _ = O.TangentOracle(host).jvp(u, v)
    assert np.array_equal(r, O.Oracle(host).residual(u))


def _fd_errors(host, u, seed):
    orc = O.Oracle(host)
    rng = np.random.default_rng(seed)
    v = rng.standard_normal(u.shape) * np.abs(u).max() * 1e-2
    _, jv = O.TangentOracle(host).jvp(u, v)
    return [O.rel2(jv, (orc.residual(u + h * v) - orc.residual(u - h * v)) / (2 * h)) for h in STEPS]


def test_tangent_matches_central_differences(case):
    host, u = case
    lf_euler = host.cfg.law == 1 and host.cfg.numerical_flux == 0 and host.cfg.half_lambda > 0
    # Lax-Friedrichs on a smooth Euler state: inner and outer states nearly
    # coincide, so max(|V.n|) and max(c) sit near their switching points at
    # many facet nodes and the differences straddle kinks; without the
    # dissipation (next test) the agreement is 1e-6 or better
    assert min(_fd_errors(host, u, 4)) < (1e-4 if lf_euler else 1e-6)


@pytest.mark.parametrize("name", ["vortex_tri_modal", "euler_tri_std", "tgv_tet_modal", "tgv_tet_p5"])
def test_tangent_without_dissipation(name):
    host, u = cases.make(name)
    host.cfg.half_lambda = 0.0  # a = 0: the interface flux is smooth
    assert min(_fd_errors(host, u, 4)) < 1e-6


@pytest.mark.parametrize("name", ["adv_tri_modal", "adv_tet_fd"])
def test_linear_residual_tangent_is_the_residual(name):
    host, u = cases.make(name)
    rng = np.random.default_rng(5)
    v = rng.standard_normal(u.shape)
    _, jv = O.TangentOracle(host).jvp(u, v)
    assert O.rel2(jv, O.Oracle(host).residual(v)) < 1e-14


@pytest.mark.parametrize("scheme", [0, 1])
def test_trajectory_tangent(scheme):
    host, u = cases.make("vortex_tri_modal")
    orc = O.Oracle(host)
    rng = np.random.default_rng(6)
    v = rng.standard_normal(u.shape) * 1e-2
    dt, n = 2e-3, 3
    uT, w = O.TangentOracle(host).rk_jvp(u, v, n, dt, scheme)
    assert np.array_equal(uT, orc.rk_steps(u, n, dt, scheme))
    errs = [O.rel2(w, (orc.rk_steps(u + h * v, n, dt, scheme) - orc.rk_steps(u - h * v, n, dt, scheme)) / (2 * h))
            for h in STEPS]
    assert min(errs) < 1e-6, errs
