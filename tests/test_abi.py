"""The C-ABI library without a GPU: it builds for sm_103a, loads, exports
every function include/sse_gb300.h declares, agrees with the ctypes struct
layouts, and rejects invalid arguments before touching the device."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import cases

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "sse_gb300.h")


@pytest.fixture(scope="module")
def lib(pkg):
    pkg.build.build()
    return pkg.load_library()


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sse_[a-z_]+)\s*\(", text)))


def test_exports_every_declared_symbol(pkg, lib):
    out = subprocess.run(["nm", "-D", "--defined-only", pkg.gb300.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (sse_\w+)", out))
    missing = [f for f in declared_functions() if f not in exported]
    assert not missing, missing
    assert set(pkg.gb300.EXPORTED) <= exported


def test_struct_layouts(pkg, lib):
    abi = pkg.abi
    sizes = (C.c_int32 * 6)()
    assert lib.sse_struct_sizes(sizes) == 6
    assert list(sizes) == [C.sizeof(abi.SseConfig), C.sizeof(abi.SseCsc),
                           C.sizeof(abi.SseOperators), C.sizeof(abi.SseGeometry),
                           C.sizeof(abi.SseMetricOperators), C.sizeof(abi.SseGeometricFactorsOut)]
    assert lib.sse_abi_version() == 1


def _create(pkg, lib, host):
    h = C.c_void_p()
    rc = lib.sse_create(C.byref(host.cfg), C.byref(host.ops), C.byref(host.geo), C.byref(h))
    return rc, lib.sse_create_error().decode(), h


def test_rejects_invalid_arguments_on_host(pkg, lib):
    abi = pkg.abi
    host, _ = cases.make("vortex_tri_modal")
    h = C.c_void_p()
    assert lib.sse_create(None, C.byref(host.ops), C.byref(host.geo), C.byref(h)) == abi.SSE_ERR_INVALID_ARGUMENT
    # out-of-range connectivity
    saved = host.mapP.copy()
    host.mapP[0, 0] = host.N_f * host.N_e + 1
    rc, msg, h = _create(pkg, lib, host)
    host.mapP[:] = saved
    assert rc == abi.SSE_ERR_INVALID_ARGUMENT and "mapP" in msg and not h.value
    # unsupported law / size combination
    host.cfg.n_c = 3
    rc, msg, _ = _create(pkg, lib, host)
    host.cfg.n_c = 4
    assert rc == abi.SSE_ERR_UNSUPPORTED
    # an empty mesh (no elements) is rejected on the host
    ne = host.cfg.n_e
    host.cfg.n_e = 0
    rc, msg, h0 = _create(pkg, lib, host)
    host.cfg.n_e = ne
    assert rc == abi.SSE_ERR_INVALID_ARGUMENT and not h0.value
    # inconsistent facet count
    host.cfg.nodes_per_face += 1
    rc, msg, _ = _create(pkg, lib, host)
    host.cfg.nodes_per_face -= 1
    assert rc == abi.SSE_ERR_INVALID_ARGUMENT
    # corrupted CSC row index
    host.S[0].rowval[0] = host.N_q + 5
    rc, msg, _ = _create(pkg, lib, host)
    host.S[0].rowval[0] = 1
    assert rc == abi.SSE_ERR_INVALID_ARGUMENT and "row index" in msg
    # modal index map that repeats a mode
    sig = host.vdm_sigma
    flat = sig.reshape(-1)
    nz = np.nonzero(flat)[0]
    old = flat[nz[1]]
    flat[nz[1]] = flat[nz[0]]
    rc, msg, _ = _create(pkg, lib, host)
    flat[nz[1]] = old
    assert rc == abi.SSE_ERR_INVALID_ARGUMENT and "sigma" in msg


def test_null_handle_calls(pkg, lib):
    abi = pkg.abi
    assert lib.sse_residual(None, None, None, 0.0, 0) == abi.SSE_ERR_INVALID_ARGUMENT
    assert lib.sse_residual_vjp(None, None, None, None, 0) == abi.SSE_ERR_INVALID_ARGUMENT
    assert lib.sse_rk_record(None, None, 1, 1e-3, 0, 0, None, 0) == abi.SSE_ERR_INVALID_ARGUMENT
    assert lib.sse_rk_adjoint(None, None, None, None, 0) == abi.SSE_ERR_INVALID_ARGUMENT
    assert lib.sse_destroy(None) == abi.SSE_OK
    assert lib.sse_last_error(None) == b"null handle"


def test_product_has_no_cpu_fallback(pkg):
    """The package never imports the oracle and fails loudly without its library."""
    pkg_dir = os.path.join(ROOT, "cloud.jl_gb300")
    for f in os.listdir(pkg_dir):
        if f.endswith(".py"):
            assert "oracle" not in open(os.path.join(pkg_dir, f)).read().replace("Oracle", "")
    saved = pkg.gb300._lib
    pkg.gb300._lib = None
    try:
        with pytest.raises(RuntimeError, match="missing"):
            pkg.gb300.load_library(os.path.join(ROOT, "does-not-exist.so"))
    finally:
        pkg.gb300._lib = saved


def test_geometric_factors_rejects_invalid_arguments(pkg, lib):
    """sse_geometric_factors validates its operators and sizes before it
    touches the device."""
    abi = pkg.abi
    ops = abi.SseMetricOperators()
    res = abi.SseGeometricFactorsOut()
    xyz = (C.c_void_p * 3)()
    assert lib.sse_geometric_factors(None, 4, xyz, C.byref(res), abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    ops.d = 4
    assert lib.sse_geometric_factors(C.byref(ops), 4, xyz, C.byref(res), abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    assert "d must be" in lib.sse_create_error().decode()
    ops.d, ops.metrics = 3, 7
    assert lib.sse_geometric_factors(C.byref(ops), 4, xyz, C.byref(res), abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    ops.metrics = abi.SSE_CONSERVATIVE_CURL_METRICS
    ops.n_map, ops.n_q, ops.n_f, ops.num_faces = 10, 27, 30, 4    # 30 facet nodes on 4 faces
    assert lib.sse_geometric_factors(C.byref(ops), 4, xyz, C.byref(res), abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    assert "sizes" in lib.sse_create_error().decode()
    # a complete set of matrices but no degree N+1 element for the Tet curl form
    ra = pkg.reference.reference_approximation("ModalTensor", "Tet", 2, mapping_degree=2)
    mo = pkg.mesh.metric_operators(ra, "Exact", False)
    keep = [np.asfortranarray(a) for a in (*mo.Drst, mo.Vq, mo.Vf, *mo.nrstJ)]
    dp = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    ops.n_map, ops.n_q, ops.n_f = mo.Vq.shape[1], mo.Vq.shape[0], mo.Vf.shape[0]
    for m in range(3):
        ops.Drst[m], ops.nrstJ[m] = dp(keep[m]), dp(keep[5 + m])
    ops.Vq, ops.Vf = dp(keep[3]), dp(keep[4])
    x = np.zeros((4, ops.n_map))
    xyz = (C.c_void_p * 3)(x.ctypes.data, x.ctypes.data, x.ctypes.data)
    assert lib.sse_geometric_factors(C.byref(ops), 4, xyz, C.byref(res), abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    assert "n_curl" in lib.sse_create_error().decode()
    # projection is defined for exact metrics only
    ops.metrics, ops.project_jacobian = abi.SSE_EXACT_METRICS, 1
    assert lib.sse_geometric_factors(C.byref(ops), 4, xyz, C.byref(res), abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    assert "project" in lib.sse_create_error().decode()
    # outputs are required
    ops.project_jacobian = 0
    assert lib.sse_geometric_factors(C.byref(ops), 4, xyz, C.byref(res), abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    assert "output" in lib.sse_create_error().decode()


def test_project_function_rejects_invalid_arguments(pkg, lib):
    abi = pkg.abi
    x = np.zeros(16)
    p = C.c_void_p(x.ctypes.data)
    assert lib.sse_project_function(0, 4, 1, 1, p, p, p, p, p, abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    assert lib.sse_project_function(5, 4, 1, 1, p, p, p, p, p, abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    assert "n_p" in lib.sse_create_error().decode()
    assert lib.sse_project_function(2, 4, 1, 1, None, p, p, p, p, abi.SSE_HOST) == abi.SSE_ERR_INVALID_ARGUMENT
    assert lib.sse_project_function(2, 4, 1, 1, p, p, p, p, p, 7) == abi.SSE_ERR_INVALID_ARGUMENT
