"""ctypes front end of the C oracle (oracle/sse_oracle.c).

TEST INFRASTRUCTURE ONLY.  The oracle restates the reference's CPU residual
(src/Solvers/*.jl, src/ConservationLaws/*.jl, src/MatrixFreeOperators/
warped_product_*.jl) and is used by tests/, __graft_entry__.smoke() and the
cpu_baseline / --impl reference legs of bench.py to check and time the CUDA
library.  The product never imports this module.

Two builds exist: the default one (no floating-point contraction beyond the
explicit fma() calls that mirror the reference's @muladd) and an ``fma``
variant compiled with contraction enabled.  Both are valid FP64 evaluations
of the same code; their difference measures the round-off floor of a
residual on a given input, which calibrates the parity tolerance.
"""
from __future__ import annotations

import ctypes as C
import os
import platform
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sse_oracle.c")
HDR = os.path.join(HERE, "..", "include", "sse_gb300.h")
BUILD = os.path.join(HERE, "_build")
VARIANTS = {
    "default": ["-ffp-contract=off"],
    "fma": ["-ffp-contract=fast"] + (["-mfma"] if platform.machine() in ("x86_64", "AMD64") else []),
}


def lib_path(variant: str = "default") -> str:
    return os.path.join(BUILD, f"libsse_oracle_{variant}.so")


def build(force: bool = False, variant: str = "default") -> str:
    """Compile the oracle with gcc -O3 -fopenmp (no fast-math)."""
    os.makedirs(BUILD, exist_ok=True)
    out = lib_path(variant)
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR))
    if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    cmd = ["gcc", "-O3", "-std=c99", "-fPIC", "-shared", "-fopenmp", *VARIANTS[variant],
           SRC, "-o", out + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


_libs: dict = {}


def lib(variant: str = "default"):
    if variant not in _libs:
        L = C.CDLL(build(variant=variant))
        L.oracle_create.restype = C.c_void_p
        L.oracle_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_destroy.argtypes = [C.c_void_p]
        L.oracle_residual.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_nodal_values.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_rk_steps.argtypes = [C.c_void_p, C.c_void_p, C.c_int, C.c_double, C.c_int]
        L.oracle_conservation_residual.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p]
        L.oracle_threads.restype = C.c_int
        _libs[variant] = L
    return _libs[variant]


def _ptr(a):
    return C.c_void_p(a.ctypes.data)


class Oracle:
    """CPU residual over the same HostArrays the CUDA library consumes."""

    def __init__(self, host, nthreads: int | None = None, variant: str = "default"):
        self.L = lib(variant)
        self.host = host
        self.nthreads = nthreads or self.L.oracle_threads()
        self.h = self.L.oracle_create(C.byref(host.cfg), C.byref(host.ops), C.byref(host.geo),
                                      self.nthreads)

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_destroy(self.h)
            self.h = None

    def residual(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        assert u.shape == self.host.state_shape
        dudt = np.empty_like(u)
        self.L.oracle_residual(self.h, _ptr(u), _ptr(dudt))
        return dudt

    def nodal_values(self, u: np.ndarray):
        u = np.ascontiguousarray(u, dtype=np.float64)
        h = self.host
        u_q = np.empty((h.N_e, h.N_c, h.N_q))
        u_f = np.empty((h.N_c, h.N_e, h.N_f))
        self.L.oracle_nodal_values(self.h, _ptr(u), _ptr(u_q), _ptr(u_f))
        return u_q, u_f

    def rk_steps(self, u: np.ndarray, n_steps: int, dt: float, scheme: int = 0) -> np.ndarray:
        u = np.array(u, dtype=np.float64, order="C", copy=True)
        self.L.oracle_rk_steps(self.h, _ptr(u), n_steps, dt, scheme)
        return u

    def conservation_residual(self, u: np.ndarray, dudt: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        dudt = np.ascontiguousarray(dudt, dtype=np.float64)
        out = np.zeros(self.host.N_c + 1)
        self.L.oracle_conservation_residual(self.h, _ptr(u), _ptr(dudt), _ptr(out))
        return out


TANGENT_SRC = os.path.join(HERE, "sse_oracle_tangent.cpp")


def build_tangent(force: bool = False) -> str:
    """Compile the dual-number build of the same oracle source (g++ -O3
    -fopenmp, no contraction beyond the explicit fma() calls)."""
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libsse_oracle_tangent.so")
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR), os.path.getmtime(TANGENT_SRC))
    if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           TANGENT_SRC, "-o", out + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


_tangent_lib = None


def tangent_lib():
    global _tangent_lib
    if _tangent_lib is None:
        L = C.CDLL(build_tangent())
        L.oracle_tangent_create.restype = C.c_void_p
        L.oracle_tangent_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
        L.oracle_tangent_destroy.argtypes = [C.c_void_p]
        L.oracle_tangent_residual.argtypes = [C.c_void_p] * 5
        L.oracle_tangent_rk_steps.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int,
                                              C.c_double, C.c_int]
        _tangent_lib = L
    return _tangent_lib


class TangentOracle:
    """Forward-mode derivatives of the oracle: J(u) v and the tangent of a
    whole fixed-step trajectory (dual numbers through sse_oracle.c)."""

    def __init__(self, host, nthreads: int | None = None):
        self.L = tangent_lib()
        self.host = host
        self.h = self.L.oracle_tangent_create(C.byref(host.cfg), C.byref(host.ops), C.byref(host.geo),
                                              nthreads or lib().oracle_threads())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_tangent_destroy(self.h)
            self.h = None

    def jvp(self, u: np.ndarray, v: np.ndarray):
        """(R(u), J(u) v)."""
        u = np.ascontiguousarray(u, dtype=np.float64)
        v = np.ascontiguousarray(v, dtype=np.float64)
        assert u.shape == v.shape == self.host.state_shape
        r, jv = np.empty_like(u), np.empty_like(u)
        self.L.oracle_tangent_residual(self.h, _ptr(u), _ptr(v), _ptr(r), _ptr(jv))
        return r, jv

    def rk_jvp(self, u: np.ndarray, v: np.ndarray, n_steps: int, dt: float, scheme: int = 0):
        """(u(T), (du(T)/du(0)) v)."""
        u = np.array(u, dtype=np.float64, order="C", copy=True)
        v = np.array(v, dtype=np.float64, order="C", copy=True)
        self.L.oracle_tangent_rk_steps(self.h, _ptr(u), _ptr(v), n_steps, dt, scheme)
        return u, v


EXTENDED_SRC = os.path.join(HERE, "sse_oracle_extended.cpp")


def build_extended(force: bool = False) -> str:
    """Compile the extended-precision (long double) build of the same
    oracle source (g++ -O3 -fopenmp, no contraction beyond explicit fma())."""
    os.makedirs(BUILD, exist_ok=True)
    out = os.path.join(BUILD, "libsse_oracle_extended.so")
    newest = max(os.path.getmtime(SRC), os.path.getmtime(HDR), os.path.getmtime(EXTENDED_SRC))
    if not force and os.path.exists(out) and os.path.getmtime(out) >= newest:
        return out
    cmd = ["g++", "-O3", "-std=c++17", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off",
           EXTENDED_SRC, "-o", out + ".tmp", "-lm"]
    subprocess.run(cmd, check=True)
    os.replace(out + ".tmp", out)
    return out


_extended_lib = None


class ExtendedOracle:
    """The oracle's residual evaluated in long double (the reference for
    measuring how far an FP64 residual is from the exact one)."""

    def __init__(self, host, nthreads: int | None = None):
        global _extended_lib
        if _extended_lib is None:
            L = C.CDLL(build_extended())
            L.oracle_extended_create.restype = C.c_void_p
            L.oracle_extended_create.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int]
            L.oracle_extended_destroy.argtypes = [C.c_void_p]
            L.oracle_extended_residual.argtypes = [C.c_void_p] * 3
            L.oracle_extended_digits.restype = C.c_int
            _extended_lib = L
        self.L = _extended_lib
        self.host = host
        self.digits = self.L.oracle_extended_digits()
        self.h = self.L.oracle_extended_create(C.byref(host.cfg), C.byref(host.ops), C.byref(host.geo),
                                               nthreads or lib().oracle_threads())

    def __del__(self):
        if getattr(self, "h", None):
            self.L.oracle_extended_destroy(self.h)
            self.h = None

    def residual(self, u: np.ndarray) -> np.ndarray:
        u = np.ascontiguousarray(u, dtype=np.float64)
        out = np.empty_like(u)
        self.L.oracle_extended_residual(self.h, _ptr(u), _ptr(out))
        return out


def rel2(got, want) -> float:
    """Whole-vector relative error ||got - want||_2 / ||want||_2."""
    got = np.asarray(got, dtype=np.float64)
    want = np.asarray(want, dtype=np.float64)
    return float(np.linalg.norm(got - want) / max(np.linalg.norm(want), 1e-300))


def roundoff_floor(host, u) -> float:
    """rel2 between the two oracle builds on the same input."""
    a = Oracle(host).residual(u)
    b = Oracle(host, variant="fma").residual(u)
    return rel2(b, a)
