"""Pin the oracle to the reference's own golden values (test/runtests.jl,
extracted to tests/golden/reference_goldens.json by
tests/golden/extract_reference_goldens.py).  Same tolerance as the
reference's tests: 1e-10 absolute."""
import json
import os

import numpy as np
import pytest

import reference_scenarios as RS
from oracle.oracle import Oracle

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "reference_goldens.json")))
TOL = GOLD["tol"]


def test_advection_2d_modal_tensor_tri_golden():
    sc = RS.advection_2d()
    host = sc["host"]
    o = Oracle(host)
    u = sc["u0"].copy()
    cons, energy = [], []
    for step in range(0, sc["steps"] + 1, sc["save_every"]):
        if step:
            u = o.rk_steps(u, sc["save_every"], sc["dt"], 0)
        du = o.residual(u)
        cons.append(o.conservation_residual(u, du)[0])
        energy.append(RS.energy_rate_wa(host, u, du))
    l2 = RS.l2_error(sc["sd"], u, sc["exact"])[0]
    g = GOLD["advection_2d_modal_tensor_tri"]
    assert abs(l2 - g["l2"]) < TOL, (l2, g["l2"])
    assert max(abs(c) for c in cons) < TOL
    assert max(abs(e) for e in energy) < TOL


def test_euler_vortex_2d_modal_tensor_tri_golden():
    sc = RS.euler_vortex_2d()
    host = sc["host"]
    o = Oracle(host)
    E0 = RS.conserved_totals(host, sc["u0"])
    u = o.rk_steps(sc["u0"], sc["steps"], sc["dt"], 0)
    l2 = RS.l2_error(sc["sd"], u, sc["exact"])
    g = GOLD["euler_vortex_2d_modal_tensor_tri_fd_lf"]
    assert np.abs(l2 - np.array(g["l2"])).max() < TOL, (l2, g["l2"])
    assert np.abs(RS.conserved_totals(host, u) - E0).max() < TOL
