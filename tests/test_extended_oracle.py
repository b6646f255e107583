"""The extended-precision (long double) build of the oracle: it carries
more mantissa bits than FP64 and agrees with the FP64 oracle to the FP64
round-off floor, so it serves as the reference the FP64 residuals are
measured against (their distance to it is the error of an FP64 evaluation,
cancellation included)."""
import pytest

import cases
from oracle.oracle import ExtendedOracle, Oracle, rel2, roundoff_floor


@pytest.mark.parametrize("name", ["vortex_tri_modal", "tgv_tet_modal", "adv_tri_modal", "euler_tet_std"])
def test_extended_oracle_agrees_with_fp64_to_the_floor(name):
    host, u = cases.make(name)
    ext = ExtendedOracle(host)
    assert ext.digits > 53
    r64 = Oracle(host).residual(u)
    rx = ext.residual(u)
    floor = roundoff_floor(host, u)
    assert rel2(r64, rx) <= max(4.0 * floor, 1e-15)
