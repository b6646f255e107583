"""save_callback around the device time loop: sol_<n>.jld2 files written
from the snapshot hook hold the states and residuals of stepping on the GPU."""
import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu


def test_save_callback_writes_the_device_trajectory(gpu_lib, pkg, tmp_path):
    J = pkg.jld2
    host, u0 = cases.make("vortex_tri_modal")
    G = pkg.GB300Solver(host)
    dt = 1e-3
    path = str(tmp_path / "run") + "/"
    J.new_path(path)
    J.save_object(path + "time_steps.jld2", np.zeros(0, dtype=np.int64))
    u, t = J.save_callback(G, path, u0, n_steps=7, dt=dt, interval=3)
    assert list(J.load_time_steps(path)) == [0, 3, 6, 7]
    assert t == pytest.approx(7 * dt)
    w = u0.copy()
    done = 0
    for step in (0, 3, 6, 7):
        if step > done:
            G.rk_steps(w, step - done, dt)
        done = step
        us, dus, ts = J.load_solution(path, step, load_du=True)
        assert ts == pytest.approx(step * dt)
        assert np.array_equal(us, w)
        assert np.array_equal(dus, G.residual(w))
    assert np.array_equal(u, w)
    log = open(path + "screen.txt").read().splitlines()
    assert [ln.split()[3] for ln in log] == ["0", "3", "6", "7"]
