"""GB300 backend: the ``GB300 <: AbstractParallelism`` drop-in.

``semidiscretize(..., parallelism=GB300())`` builds the reference's operator
structs on the host (``HostArrays``), hands them once to the C-ABI library
``libsse_gb300.so`` and returns an ``ODEProblem`` whose right-hand side
``semi_discrete_residual(dudt, u, solver, t)`` runs entirely on the GPU
(Solvers.jl:429-514).  There is no CPU path: if the library is missing or
no CUDA device is present, every call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

from . import abi
from .solver import HostArrays, initialize

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libsse_gb300.so")

EXPORTED = ["sse_abi_version", "sse_create", "sse_destroy", "sse_residual",
            "sse_residual_static_scratch", "sse_nodal_values",
            "sse_rk_steps", "sse_rk_steps_snapshots", "sse_residual_vjp", "sse_rk_record",
            "sse_rk_adjoint", "sse_rk_record_binomial", "sse_binomial_schedule",
            "sse_conservation_residual", "sse_set_precision", "sse_set_stream",
            "sse_phase_timings", "sse_struct_sizes", "sse_measure_fma_peaks", "sse_last_error",
            "sse_create_error", "sse_geometric_factors", "sse_project_function",
            "sse_energy_residual", "sse_kernel_path", "sse_set_kernel_path"]

_lib = None


class SSEError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"sse status {code}: {msg}")
        self.code = code


def load_library(path: str | None = None):
    """Load libsse_gb300.so (built by build.build()); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIB_PATH
    if not os.path.exists(path):
        raise RuntimeError(f"{path} is missing: build the CUDA library first (build.build())")
    L = C.CDLL(path)
    vp, i32, dp = C.c_void_p, C.c_int32, C.c_double
    L.sse_abi_version.restype = i32
    L.sse_create.argtypes = [vp, vp, vp, C.POINTER(vp)]
    L.sse_create.restype = i32
    L.sse_destroy.argtypes = [vp]
    L.sse_destroy.restype = i32
    L.sse_residual.argtypes = [vp, vp, vp, dp, i32]
    L.sse_residual.restype = i32
    L.sse_residual_static_scratch.argtypes = [vp, vp, vp]
    L.sse_residual_static_scratch.restype = i32
    L.sse_nodal_values.argtypes = [vp, vp, vp, vp, i32]
    L.sse_nodal_values.restype = i32
    L.sse_rk_steps.argtypes = [vp, vp, i32, dp, i32, C.POINTER(dp), i32]
    L.sse_rk_steps.restype = i32
    L.sse_rk_steps_snapshots.argtypes = [vp, vp, i32, dp, i32, i32, vp, vp, C.POINTER(dp), i32]
    L.sse_rk_steps_snapshots.restype = i32
    L.sse_residual_vjp.argtypes = [vp, vp, vp, vp, i32]
    L.sse_residual_vjp.restype = i32
    L.sse_rk_record.argtypes = [vp, vp, i32, dp, i32, i32, C.POINTER(dp), i32]
    L.sse_rk_record.restype = i32
    L.sse_rk_adjoint.argtypes = [vp, vp, vp, vp, i32]
    L.sse_rk_adjoint.restype = i32
    L.sse_rk_record_binomial.argtypes = [vp, vp, i32, dp, i32, i32, C.POINTER(dp), i32]
    L.sse_rk_record_binomial.restype = i32
    L.sse_binomial_schedule.argtypes = [i32, i32, C.POINTER(C.c_int64), C.POINTER(i32)]
    L.sse_binomial_schedule.restype = i32
    L.sse_conservation_residual.argtypes = [vp, vp, vp, vp, i32]
    L.sse_conservation_residual.restype = i32
    L.sse_energy_residual.argtypes = [vp, vp, vp, vp, i32]
    L.sse_energy_residual.restype = i32
    L.sse_set_precision.argtypes = [vp, i32]
    L.sse_set_precision.restype = i32
    L.sse_set_stream.argtypes = [vp, vp]
    L.sse_set_stream.restype = i32
    L.sse_phase_timings.argtypes = [vp, vp, i32, vp]
    L.sse_phase_timings.restype = i32
    L.sse_kernel_path.argtypes = [vp]
    L.sse_kernel_path.restype = i32
    L.sse_set_kernel_path.argtypes = [vp, i32]
    L.sse_set_kernel_path.restype = i32
    L.sse_measure_fma_peaks.argtypes = [vp]
    L.sse_measure_fma_peaks.restype = i32
    L.sse_struct_sizes.argtypes = [vp]
    L.sse_struct_sizes.restype = i32
    L.sse_last_error.argtypes = [vp]
    L.sse_last_error.restype = C.c_char_p
    L.sse_create_error.restype = C.c_char_p
    L.sse_geometric_factors.argtypes = [vp, C.c_int64, vp, vp, i32]
    L.sse_geometric_factors.restype = i32
    L.sse_project_function.argtypes = [i32, i32, i32, C.c_int64, vp, vp, vp, vp, vp, i32]
    L.sse_project_function.restype = i32
    _lib = L
    return L


def _addr(x):
    """Raw address of a numpy array or a torch tensor (host or device)."""
    if isinstance(x, np.ndarray):
        assert x.dtype == np.float64 and x.flags.c_contiguous
        return C.c_void_p(x.ctypes.data), abi.SSE_HOST
    # torch tensor
    assert x.dtype.__repr__() == "torch.float64" and x.is_contiguous()
    return C.c_void_p(x.data_ptr()), (abi.SSE_DEVICE if x.is_cuda else abi.SSE_HOST)


class GB300Solver:
    """``Solver{..., GB300}``: owns one library handle."""

    def __init__(self, host: HostArrays):
        self.host = host
        self.L = load_library()
        h = C.c_void_p()
        rc = self.L.sse_create(C.byref(host.cfg), C.byref(host.ops), C.byref(host.geo), C.byref(h))
        if rc != abi.SSE_OK:
            raise SSEError(rc, self.L.sse_create_error().decode())
        self.h = h

    def close(self):
        if getattr(self, "h", None):
            self.L.sse_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != abi.SSE_OK:
            raise SSEError(rc, self.L.sse_last_error(self.h).decode())

    def residual(self, u, dudt=None, t: float = 0.0):
        if dudt is None:
            dudt = np.empty_like(u) if isinstance(u, np.ndarray) else u.new_empty(u.shape)
        pu, mu = _addr(u)
        pd, md = _addr(dudt)
        assert mu == md, "u and dudt must live in the same memory"
        self._check(self.L.sse_residual(self.h, pu, pd, t, mu))
        return dudt

    def nodal_values(self, u):
        h = self.host
        if isinstance(u, np.ndarray):
            u_q = np.empty((h.N_e, h.N_c, h.N_q))
            u_f = np.empty((h.N_c, h.N_e, h.N_f))
        else:
            u_q = u.new_empty((h.N_e, h.N_c, h.N_q))
            u_f = u.new_empty((h.N_c, h.N_e, h.N_f))
        pu, mu = _addr(u)
        self._check(self.L.sse_nodal_values(self.h, pu, _addr(u_q)[0], _addr(u_f)[0], mu))
        return u_q, u_f

    def rk_steps(self, u, n_steps: int, dt: float, scheme: int = abi.SSE_CARPENTER_KENNEDY_2N54,
                 t: float = 0.0) -> float:
        pu, mu = _addr(u)
        tt = C.c_double(t)
        self._check(self.L.sse_rk_steps(self.h, pu, n_steps, dt, scheme, C.byref(tt), mu))
        return tt.value

    def rk_steps_snapshots(self, u, n_steps: int, dt: float, every: int,
                           scheme: int = abi.SSE_CARPENTER_KENNEDY_2N54, with_residuals: bool = False,
                           t: float = 0.0):
        """``rk_steps`` with the ``save_callback`` hook: returns (t, snapshots,
        residuals) with the state (and its residual) after every ``every``-th
        step, in the memory kind of ``u``."""
        k = n_steps // every
        if k == 0:
            t = self.rk_steps(u, n_steps, dt, scheme, t)
            shape = (0,) + tuple(u.shape)
            empty = np.empty(shape) if isinstance(u, np.ndarray) else u.new_empty(shape)
            return t, empty, (empty if with_residuals else None)
        if isinstance(u, np.ndarray):
            snaps = np.empty((k,) + u.shape)
            res = np.empty((k,) + u.shape) if with_residuals else None
        else:
            snaps = u.new_empty((k,) + tuple(u.shape))
            res = u.new_empty((k,) + tuple(u.shape)) if with_residuals else None
        pu, mu = _addr(u)
        ps = _addr(snaps)[0]
        pr = _addr(res)[0] if res is not None else C.c_void_p(0)
        tt = C.c_double(t)
        self._check(self.L.sse_rk_steps_snapshots(self.h, pu, n_steps, dt, scheme, every, ps, pr,
                                                  C.byref(tt), mu))
        return tt.value, snaps, res

    def residual_vjp(self, u, lam, mu=None):
        """(dR/du)^T lam at u: the discrete adjoint of ``residual``."""
        if mu is None:
            mu = np.empty_like(u) if isinstance(u, np.ndarray) else u.new_empty(u.shape)
        pu, mu_u = _addr(u)
        pl, mu_l = _addr(lam)
        pm, mu_m = _addr(mu)
        assert mu_u == mu_l == mu_m, "u, lam and mu must live in the same memory"
        self._check(self.L.sse_residual_vjp(self.h, pu, pl, pm, mu_u))
        return mu

    def rk_record(self, u, n_steps: int, dt: float, scheme: int = abi.SSE_CARPENTER_KENNEDY_2N54,
                  checkpoint_every: int = 0, t: float = 0.0) -> float:
        """``rk_steps`` that records checkpoints for ``rk_adjoint``."""
        pu, mu = _addr(u)
        tt = C.c_double(t)
        self._check(self.L.sse_rk_record(self.h, pu, n_steps, dt, scheme, checkpoint_every,
                                         C.byref(tt), mu))
        return tt.value

    def rk_record_binomial(self, u, n_steps: int, dt: float, scheme: int = abi.SSE_CARPENTER_KENNEDY_2N54,
                           n_checkpoints: int = 0, t: float = 0.0) -> float:
        """``rk_steps`` that records for ``rk_adjoint`` on the binomial
        (revolve) schedule with ``n_checkpoints`` checkpoints (0: as many as
        fit)."""
        pu, mu = _addr(u)
        tt = C.c_double(t)
        self._check(self.L.sse_rk_record_binomial(self.h, pu, n_steps, dt, scheme, n_checkpoints,
                                                  C.byref(tt), mu))
        return tt.value

    def rk_adjoint(self, lam_T, lam_0=None) -> dict:
        """(du(T)/du(0))^T lam_T for the last ``rk_record``; returns
        {"lam_0", "segments", "checkpoint_every", "bytes", "recomputed"}."""
        if lam_0 is None:
            lam_0 = np.empty_like(lam_T) if isinstance(lam_T, np.ndarray) else lam_T.new_empty(lam_T.shape)
        pl, ml = _addr(lam_T)
        p0, m0 = _addr(lam_0)
        assert ml == m0
        info = np.zeros(4)
        self._check(self.L.sse_rk_adjoint(self.h, pl, p0, C.c_void_p(info.ctypes.data), ml))
        return {"lam_0": lam_0, "segments": int(info[0]), "checkpoint_every": int(info[1]),
                "bytes": int(info[2]), "recomputed": int(info[3])}

    def conservation_residual(self, u, dudt) -> np.ndarray:
        out = np.zeros(self.host.N_c + 1)
        pu, mu = _addr(u)
        pd, md = _addr(dudt)
        assert mu == md
        self._check(self.L.sse_conservation_residual(self.h, pu, pd, C.c_void_p(out.ctypes.data), mu))
        return out

    def energy_residual(self, u, dudt) -> np.ndarray:
        """EnergyConservationAnalysis residual: sum_k u' M_k dudt per component
        with the mass solver's own mass matrix (sse_energy_residual)."""
        out = np.zeros(self.host.N_c)
        pu, mu = _addr(u)
        pd, md = _addr(dudt)
        assert mu == md
        self._check(self.L.sse_energy_residual(self.h, pu, pd, C.c_void_p(out.ctypes.data), mu))
        return out

    def set_precision(self, precision: int):
        self._check(self.L.sse_set_precision(self.h, precision))

    def set_stream(self, stream_handle: int):
        self._check(self.L.sse_set_stream(self.h, C.c_void_p(stream_handle)))

    def kernel_path(self) -> int:
        """SSE_PATH_TWO_PHASE or SSE_PATH_ONE_KERNEL (sse_kernel_path)."""
        r = self.L.sse_kernel_path(self.h)
        if r < 0:
            self._check(r)
        return r

    def set_kernel_path(self, path: int):
        self._check(self.L.sse_set_kernel_path(self.h, path))

    def phase_timings(self, u_dev, n_iter: int) -> np.ndarray:
        out = np.zeros(3)
        self._check(self.L.sse_phase_timings(self.h, _addr(u_dev)[0], n_iter, C.c_void_p(out.ctypes.data)))
        return out


def binomial_schedule(n_steps: int, n_checkpoints: int):
    """(extra forward steps, first checkpoint position) of the optimal
    binomial schedule (sse_binomial_schedule; host arithmetic only)."""
    L = load_library()
    extra, first = C.c_int64(0), C.c_int32(0)
    rc = L.sse_binomial_schedule(n_steps, n_checkpoints, C.byref(extra), C.byref(first))
    if rc != abi.SSE_OK:
        raise SSEError(rc, "invalid binomial schedule arguments")
    return int(extra.value), int(first.value)


def measure_fma_peaks():
    """Measured (FP64, FP32) CUDA-core FMA throughput of the device, TFLOP/s."""
    L = load_library()
    out = np.zeros(2)
    rc = L.sse_measure_fma_peaks(C.c_void_p(out.ctypes.data))
    if rc != abi.SSE_OK:
        raise SSEError(rc, "peak measurement failed")
    return float(out[0]), float(out[1])


def _fortran(a):
    """Column-major FP64 copy of a reference matrix (Julia Matrix layout)."""
    return np.asfortranarray(np.asarray(a, dtype=np.float64))


def geometric_factors(mesh, ra, metrics: str = "Exact", project_jac: bool = True, xyz=None):
    """``GeometricFactors(mesh, reference_element, metric_type)`` plus
    ``project_jacobian!`` computed on the GPU in FP64 (sse_geometric_factors).

    ``xyz`` defaults to ``mesh.xyz`` (numpy (N_e, N_map) per coordinate, the
    layout of Julia's (N_map, N_e)): the result is then a host
    ``GeometricFactors`` of numpy arrays, as the host path returns.  CUDA
    float64 tensors in ``xyz`` keep everything on the device and return the
    fields as CUDA tensors of the same shapes."""
    from .mesh import GeometricFactors, metric_operators
    L = load_library()
    mo = metric_operators(ra, metrics, project_jac)
    d = ra.d
    xyz = mesh.xyz if xyz is None else xyz
    N_e, n_map = xyz[0].shape
    keep = []

    def mat(a):
        if a is None:
            return None
        f = _fortran(a)
        keep.append(f)
        return f.ctypes.data_as(C.POINTER(C.c_double))

    ops = abi.SseMetricOperators()
    ops.d = d
    ops.metrics = abi.SSE_EXACT_METRICS if metrics == "Exact" else abi.SSE_CONSERVATIVE_CURL_METRICS
    ops.n_map = n_map
    ops.n_q = mo.Vq.shape[0]
    ops.n_f = mo.Vf.shape[0]
    ops.num_faces = mo.num_faces
    ops.n_curl = 0 if mo.N_to_N1 is None else mo.N_to_N1.shape[0]
    ops.project_jacobian = 1 if mo.project is not None else 0
    for m in range(d):
        ops.Drst[m] = mat(mo.Drst[m])
        ops.nrstJ[m] = mat(mo.nrstJ[m])
    ops.Vq = mat(mo.Vq)
    ops.Vf = mat(mo.Vf)
    if mo.N_to_N1 is not None:
        ops.N_to_Nplus1 = mat(mo.N_to_N1)
        for m in range(3):
            ops.Drst_Nplus1[m] = mat(mo.D1[m])
        ops.Vq_Nplus1 = mat(mo.Vq1)
        ops.Vf_Nplus1 = mat(mo.Vf1)
    ops.project = mat(mo.project)

    nq, nf, nfac = ops.n_q, ops.n_f, mo.num_faces
    shapes = [(N_e, nq), (N_e, d, d, nq), (N_e, nf), (N_e, nf, d), (N_e, nq, nfac, d)]
    on_device = not isinstance(xyz[0], np.ndarray)
    if on_device:
        import torch
        outs = [torch.empty(sh, dtype=torch.float64, device=xyz[0].device) for sh in shapes]
        memory = abi.SSE_DEVICE
        xs = [x.contiguous() for x in xyz]
        ptrs = (C.c_void_p * 3)(*[x.data_ptr() for x in xs], *([None] * (3 - d)))
    else:
        outs = [np.empty(sh) for sh in shapes]
        memory = abi.SSE_HOST
        xs = [np.ascontiguousarray(x, dtype=np.float64) for x in xyz]
        ptrs = (C.c_void_p * 3)(*[x.ctypes.data for x in xs], *([None] * (3 - d)))
    addr = (lambda t: t.data_ptr()) if on_device else (lambda a: a.ctypes.data)
    res = abi.SseGeometricFactorsOut(*[addr(o) for o in outs])
    rc = L.sse_geometric_factors(C.byref(ops), N_e, ptrs, C.byref(res), memory)
    if rc != abi.SSE_OK:
        raise SSEError(rc, L.sse_create_error().decode())
    return GeometricFactors(*outs)


def project_function(ra, J_q, u_q):
    """``project_function`` (Solvers.jl:396-418) on the GPU: the L2 projection
    of nodal initial data u_q (N_e, N_c, N_q numpy, or a CUDA tensor) onto
    the modal basis of ``ra`` with the element Jacobians J_q (N_e, N_q),
    by Cholesky of every element's mass matrix (sse_project_function).
    Returns u0 (N_e, N_c, N_p) in the memory of u_q."""
    L = load_library()
    if ra.V is None:
        raise ValueError("project_function on the GPU needs a modal basis (V is the identity)")
    V = _fortran(ra.V)
    W = np.ascontiguousarray(ra.W, dtype=np.float64)
    N_e, N_c, N_q = u_q.shape
    N_p = V.shape[1]
    dp = lambda a: C.c_void_p(a.ctypes.data)
    if isinstance(u_q, np.ndarray):
        J = np.ascontiguousarray(J_q, dtype=np.float64)
        uq = np.ascontiguousarray(u_q, dtype=np.float64)
        u0 = np.empty((N_e, N_c, N_p))
        rc = L.sse_project_function(N_p, N_q, N_c, N_e, dp(V), dp(W), dp(J), dp(uq), dp(u0), abi.SSE_HOST)
    else:
        import torch
        J = J_q.contiguous()
        uq = u_q.contiguous()
        u0 = torch.empty((N_e, N_c, N_p), dtype=torch.float64, device=uq.device)
        rc = L.sse_project_function(N_p, N_q, N_c, N_e, dp(V), dp(W), C.c_void_p(J.data_ptr()),
                                    C.c_void_p(uq.data_ptr()), C.c_void_p(u0.data_ptr()), abi.SSE_DEVICE)
    if rc != abi.SSE_OK:
        raise SSEError(rc, L.sse_create_error().decode())
    return u0


@dataclass
class ODEProblem:
    """``ODEProblem(semi_discrete_residual!, u0, tspan, solver)``."""
    f: object
    u0: np.ndarray
    tspan: tuple
    p: GB300Solver


def semi_discrete_residual(dudt, u, solver: GB300Solver, t: float = 0.0):
    """``semi_discrete_residual!(dudt, u, solver, t)`` on the GPU."""
    return solver.residual(u, dudt, t)


def semidiscretize(conservation_law, spatial_discretization, initial_data, form, tspan,
                   mass_matrix_solver="default") -> ODEProblem:
    """``semidiscretize(...; parallelism = GB300())`` (Solvers.jl:429-452)."""
    u0 = initialize(initial_data, spatial_discretization)
    host = HostArrays(conservation_law, spatial_discretization, form, mass_matrix_solver)
    return ODEProblem(semi_discrete_residual, u0, tuple(tspan), GB300Solver(host))
