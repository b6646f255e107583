"""ctypes mirror of include/sse_gb300.h.

The structs below must match the header byte for byte; ``check_layout``
compares their sizes with the values the compiled library reports.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

SSE_OK = 0
SSE_ERR_INVALID_ARGUMENT = 1
SSE_ERR_UNSUPPORTED = 2
SSE_ERR_CUDA = 3
SSE_ERR_NONPHYSICAL = 4
SSE_ERR_OUT_OF_MEMORY = 5

SSE_STANDARD_FORM = 0
SSE_FLUX_DIFFERENCING_FORM = 1
SSE_LINEAR_ADVECTION = 0
SSE_EULER = 1
SSE_LAX_FRIEDRICHS = 0
SSE_CENTRAL = 1
SSE_ENTROPY_CONSERVATIVE = 2
SSE_CONSERVATIVE_FLUX = 0
SSE_EC_FLUX = 1
SSE_CHANDRASHEKAR_FLUX = 2
SSE_WEIGHT_ADJUSTED = 0
SSE_DIAGONAL = 1
SSE_FP64 = 0
SSE_MIXED = 1
SSE_PATH_TWO_PHASE = 0
SSE_PATH_ONE_KERNEL = 1
SSE_HOST = 0
SSE_DEVICE = 1
SSE_CARPENTER_KENNEDY_2N54 = 0
SSE_RK4 = 1
SSE_EXACT_METRICS = 0
SSE_CONSERVATIVE_CURL_METRICS = 1

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int64)


class SseConfig(C.Structure):
    _fields_ = [("d", C.c_int32), ("n_p", C.c_int32), ("n_q", C.c_int32),
                ("n_f", C.c_int32), ("n_c", C.c_int32), ("n_e", C.c_int32),
                ("num_faces", C.c_int32), ("nodes_per_face", C.c_int32),
                ("form", C.c_int32), ("law", C.c_int32), ("numerical_flux", C.c_int32),
                ("two_point_flux", C.c_int32), ("mass_solver", C.c_int32),
                ("reserved", C.c_int32), ("half_lambda", C.c_double),
                ("gamma", C.c_double), ("a", C.c_double * 3)]


class SseCsc(C.Structure):
    _fields_ = [("m", C.c_int64), ("n", C.c_int64), ("colptr", _ip), ("rowval", _ip),
                ("nzval", _dp)]


class SseOperators(C.Structure):
    _fields_ = [("vdm_p", C.c_int32), ("vdm_m", C.c_int32 * 3), ("vdm_A", _dp),
                ("vdm_B", _dp), ("vdm_C", _dp), ("vdm_sigma_in", _ip), ("R", SseCsc),
                ("D", SseCsc * 3), ("S", SseCsc * 3), ("C", SseCsc), ("V_dense", _dp)]


class SseGeometry(C.Structure):
    _fields_ = [("BJf", _dp), ("n_f", _dp), ("mapP", _ip), ("halfWLambda", _dp),
                ("WJ", _dp), ("Lambda_q", _dp), ("halfnJf", _dp), ("halfnJq", _dp),
                ("JinvW", _dp), ("WJinv", _dp)]


class SseMetricOperators(C.Structure):
    _fields_ = [("d", C.c_int32), ("metrics", C.c_int32), ("n_map", C.c_int32),
                ("n_q", C.c_int32), ("n_f", C.c_int32), ("num_faces", C.c_int32),
                ("n_curl", C.c_int32), ("project_jacobian", C.c_int32),
                ("Drst", _dp * 3), ("Vq", _dp), ("Vf", _dp), ("nrstJ", _dp * 3),
                ("N_to_Nplus1", _dp), ("Drst_Nplus1", _dp * 3), ("Vq_Nplus1", _dp),
                ("Vf_Nplus1", _dp), ("project", _dp)]


class SseGeometricFactorsOut(C.Structure):
    _fields_ = [("J_q", C.c_void_p), ("Lambda_q", C.c_void_p), ("J_f", C.c_void_p),
                ("nJf", C.c_void_p), ("nJq", C.c_void_p)]


def dptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_dp)


def iptr(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.int64 and a.flags.c_contiguous
    return a.ctypes.data_as(_ip)


class CscArrays:
    """Host CSC arrays (1-based, Julia SparseMatrixCSC) of a dense matrix,
    dropping exact zeros like ``sparse(Matrix)``."""

    def __init__(self, dense: np.ndarray):
        dense = np.asarray(dense, dtype=np.float64)
        m, n = dense.shape
        cols, rows, vals = [], [], []
        colptr = np.zeros(n + 1, dtype=np.int64)
        colptr[0] = 1
        for j in range(n):
            nz = np.nonzero(dense[:, j] != 0.0)[0]
            rows.append(nz + 1)
            vals.append(dense[nz, j])
            colptr[j + 1] = colptr[j] + nz.size
        self.m, self.n = m, n
        self.colptr = colptr
        self.rowval = np.ascontiguousarray(np.concatenate(rows) if rows else np.zeros(0), dtype=np.int64)
        self.nzval = np.ascontiguousarray(np.concatenate(vals) if vals else np.zeros(0), dtype=np.float64)

    @property
    def nnz(self) -> int:
        return int(self.rowval.size)

    def to_dense(self) -> np.ndarray:
        out = np.zeros((self.m, self.n))
        for j in range(self.n):
            for ii in range(self.colptr[j] - 1, self.colptr[j + 1] - 1):
                out[self.rowval[ii] - 1, j] = self.nzval[ii]
        return out

    def struct(self) -> SseCsc:
        return SseCsc(self.m, self.n, iptr(self.colptr), iptr(self.rowval), dptr(self.nzval))


def empty_csc() -> SseCsc:
    return SseCsc(0, 0, None, None, None)
