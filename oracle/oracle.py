"""ctypes front end of the C oracle (oracle/sse_oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle restates the reference's CPU residual
(src/Solvers/*.jl, src/ConservationLaws/*.jl, src/MatrixFreeOperators/
warped_product_*.jl) and is used by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py to check and time the CUDA
library.  The product never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sse_oracle.c")
LIB = os.path.join(HERE, "_build", "libsse_oracle.so")


def build(force: bool = False) -> str:
    """Compile the oracle with gcc -O3 -fopenmp (no fast-math, no FP
    contraction beyond the explicit fma() calls that mirror @muladd)."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    cmd = ["gcc", "-O3", "-std=c99", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           SRC, "-o", LIB, "-lm"]
    subprocess.run(cmd, check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        path = build()
        L = C.CDLL(path)
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_residual.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_nodal_values.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_rk_steps.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int]
        L.oracle_conservation_residual.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_threads.restype = C.c_int
        _lib = L
    return _lib


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


class Oracle:
    """CPU residual over the same HostArrays the CUDA library consumes."""

    def __init__(self, host, nthreads: int | None = None):
        L = lib()
        self.host = host
        self.nthreads = nthreads or L.oracle_threads()
        self.h = L.oracle_create(C.byref(host.cfg), C.byref(host.ops), C.byref(host.geo),
                                 self.nthreads)

    def __del__(self):
        if getattr(self, "h", None):
            lib().oracle_destroy(self.h)
            self.h = None

    def residual(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.shape == self.host.state_shape
        dudt = np.empty_like(u)
        lib().oracle_residual(self.h, _ptr(u), _ptr(dudt))
        return dudt

    def nodal_values(self, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64)
        h = self.host
        u_q = np.empty((h.N_e, h.N_c, h.N_q))
        u_f = np.empty((h.N_c, h.N_e, h.N_f))
        lib().oracle_nodal_values(self.h, _ptr(u), _ptr(u_q), _ptr(u_f))
        return u_q, u_f

    def rk_steps(self, u: np.ndarray, n_steps: int, dt: float, scheme: int = 0) -> np.ndarray:
        u = np.array(u, dtype=np.float64, order="C", copy=True)
        lib().oracle_rk_steps(self.h, _ptr(u), n_steps, dt, scheme)
        return u

    def conservation_residual(self, u: np.ndarray, dudt: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        dudt = np.ascontiguousarray(dudt, dtype=np.float64)
        out = np.zeros(self.host.N_c + 1)
        lib().oracle_conservation_residual(self.h, _ptr(u), _ptr(dudt), _ptr(out))
        return out
