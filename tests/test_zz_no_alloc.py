"""sse_residual_static_scratch: the residual entry point that allocates no GPU
memory, for callers that cannot call cudaMalloc while they run (a time loop
whose memory is fixed up front, or a host framework that owns the device
memory pool).  Its two kernels pass the element nodal states through one
fixed file-scope device array instead of handle-owned buffers.

Checked through the C-ABI against sse_residual on the same handle and input
(FP64 and mixed-form handles: the entry point computes in the handle's
precision), and the FP64 result against the CPU oracle, on two calls in a
row (the second call reuses the array the first one left behind), with the
tolerances of the other parity tests.  This file is collected last so that
a run stopping at the first failure has run every other test before it; it
also passes alone in a fresh process.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from oracle.oracle import Oracle, rel2, roundoff_floor

pytestmark = pytest.mark.gpu

TOL = 1.0e-12


def _call(lib, gpu, u_dev, out_dev):
    return lib.sse_residual_static_scratch(gpu.h, C.c_void_p(u_dev.data_ptr()),
                                           C.c_void_p(out_dev.data_ptr()))


def _two_calls(lib, gpu, pkg, ud):
    """Two calls in a row into NaN-filled outputs; returns both results."""
    import torch
    outs = []
    for _ in range(2):
        got = torch.full_like(ud, float("nan"))
        torch.cuda.synchronize()                # torch's stream is not the library's
        rc = _call(lib, gpu, ud, got)
        assert rc == pkg.abi.SSE_OK, lib.sse_last_error(gpu.h).decode()
        torch.cuda.synchronize()
        outs.append(got.cpu().numpy())
    return outs


@pytest.mark.parametrize("name", ["vortex_tri_modal", "tgv_tet_modal"])
def test_static_scratch_matches_allocating_residual(gpu_lib, pkg, name):
    import torch
    host, u = cases.make(name)
    gpu = pkg.GB300Solver(host)
    lib = gpu_lib
    ud = torch.from_numpy(u).cuda()
    want = gpu.residual(ud).cpu().numpy()       # existing entry point (handle-owned scratch)
    torch.cuda.synchronize()
    oracle = Oracle(host).residual(u)
    bound = max(TOL, 4.0 * roundoff_floor(host, u))
    for call, got in enumerate(_two_calls(lib, gpu, pkg, ud)):
        assert rel2(got, want) <= TOL, call
        assert rel2(got, oracle) <= bound, call
    # a different state through the same array: still matches
    u2 = ud * 1.0001
    torch.cuda.synchronize()
    want2 = gpu.residual(u2)
    got2 = torch.empty_like(ud)
    assert _call(lib, gpu, u2, got2) == pkg.abi.SSE_OK
    torch.cuda.synchronize()
    assert rel2(got2.cpu().numpy(), want2.cpu().numpy()) <= TOL


@pytest.mark.parametrize("name", ["vortex_tri_modal", "tgv_tet_modal", "tgv_tet_exact"])
def test_static_scratch_on_a_mixed_handle(gpu_lib, pkg, name):
    """On an SSE_MIXED handle the entry point returns the mixed residual, the
    same as sse_residual on that handle, within 1e-4 of the FP64 residual."""
    import torch
    host, u = cases.make(name)
    gpu = pkg.GB300Solver(host)
    want64 = gpu.residual(u)
    gpu.set_precision(pkg.abi.SSE_MIXED)
    ud = torch.from_numpy(u).cuda()
    # the first call on this handle chooses the mixed form's reference state
    first, second = _two_calls(gpu_lib, gpu, pkg, ud)
    want = gpu.residual(ud).cpu().numpy()
    torch.cuda.synchronize()
    for got in (first, second):
        assert rel2(got, want) <= 1e-12
        assert rel2(got, want64) <= 1e-4


def test_static_scratch_rejects_meshes_beyond_capacity(gpu_lib, pkg):
    import torch
    pb = pkg.setups.tgv_tet(cells=9, p=4)       # 4374 tets: 4.9e6 doubles > 4,194,304
    host = pb.host_arrays()
    need = (host.N_q + host.N_f) * host.N_c * host.N_e * 8
    assert need > 32 * 1024 * 1024
    gpu = pkg.GB300Solver(host)
    ud = torch.from_numpy(pb.u0).cuda()
    out = torch.empty_like(ud)
    rc = _call(gpu_lib, gpu, ud, out)
    assert rc == pkg.abi.SSE_ERR_INVALID_ARGUMENT
    assert "static scratch" in gpu_lib.sse_last_error(gpu.h).decode()
    # the handle still works through the allocating entry point
    assert np.isfinite(gpu.residual(ud).cpu().numpy()).all()
