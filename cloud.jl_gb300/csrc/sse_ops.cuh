// sse_ops.cuh -- team-parallel operator applications shared by the residual
// and adjoint kernels (every per-element array lives in shared memory; a
// team of threads applies one operator to all components at once).
#pragma once

#include "sse_device.cuh"
#include "sse_kernels.cuh"

namespace sse {

// ---------------------------------------------------------------------------
// team-parallel operator applications (all NC components at once), in the
// scalar type T of the form (double: FP64 form; float: mixed form)
// ---------------------------------------------------------------------------

// Each operator below gives one thread one output node (or mode) for all NC
// components at once: the operator entry and the index arithmetic are
// loaded / computed once and feed NC independent FMA chains.  The summation
// order of every output is that of the single-component loop.

// y (NC x nq) = V x (NC x np); warped_product_2d.jl:31-55 / warped_product_3d.jl:47-84
template <typename T, int D, int NC>
__device__ void vdm_mul(const DevOps &op, const T *x, T *y, T *Z, T *W, int lane, int tpe) {
  const int np = op.np, nq = op.nq;
  if (!op.has_vdm) {
    for (int t = lane; t < NC * nq; t += tpe) y[t] = x[t];
    __syncthreads();
    return;
  }
  if (op.dense_v) {
    // dense V (multidimensional.jl:1-41): one row of V per output node
    const T *V = OpVals<T>::Vd(op);
    for (int i = lane; i < nq; i += tpe) {
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int a = 0; a < np; ++a) {
        const T v = V[i + (size_t)nq * a];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(v, x[e * np + a], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) y[e * nq + i] = acc[e];
    }
    __syncthreads();
    return;
  }
  const T *A = OpVals<T>::A(op), *B = OpVals<T>::B(op);
  const int p1 = op.p1, M1 = op.M1, M2 = op.M2;
  const float rM2 = qrcp(M2), rM3 = qrcp(op.M3 > 0 ? op.M3 : 1);
  if constexpr (D == 2) {
    // Z[e][b1][a2] = sum_b2 B[a2,b1,b2] x[sigma(b1,b2)]
    for (int s = lane; s < p1 * M2; s += tpe) {
      const int b1 = qdiv(s, rM2), a2 = s - b1 * M2;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int b2 = 0; b2 < p1 - b1; ++b2) {
        const int l = modes_index2(op, b1, b2);
        const T bv = B[a2 + M2 * (b1 + p1 * b2)];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(bv, x[e * np + l], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) Z[(e * p1 + b1) * M2 + a2] = acc[e];
    }
    __syncthreads();
    for (int s = lane; s < M1 * M2; s += tpe) {
      const int a1 = qdiv(s, rM2), a2 = s - a1 * M2;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int b1 = 0; b1 < p1; ++b1) {
        const T av = A[a1 + M1 * b1];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(av, Z[(e * p1 + b1) * M2 + a2], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) y[e * nq + M2 * a1 + a2] = acc[e];
    }
    __syncthreads();
  } else {
    const T *C = OpVals<T>::C(op);
    const int M3 = op.M3, nb12 = op.nb12;
    for (int s = lane; s < nb12 * M3; s += tpe) {
      const int q = qdiv(s, rM3), a3 = s - q * M3;
      const int b1 = op.b12[q] & 0xff, b2 = op.b12[q] >> 8;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int b3 = 0; b3 < p1 - b1 - b2; ++b3) {
        const int l = modes_index3(op, b1, b2, b3);
        const T cv = C[a3 + M3 * (b1 + p1 * (b2 + p1 * b3))];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(cv, x[e * np + l], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) Z[(e * nb12 + q) * M3 + a3] = acc[e];
    }
    __syncthreads();
    for (int s = lane; s < p1 * M2 * M3; s += tpe) {
      const int r = qdiv(s, rM3), a3 = s - r * M3, b1 = qdiv(r, rM2), a2 = r - b1 * M2;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int b2 = 0; b2 < p1 - b1; ++b2) {
        const int q = op.b12_index[b1 + p1 * b2];
        const T bv = B[a2 + M2 * (b1 + p1 * b2)];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(bv, Z[(e * nb12 + q) * M3 + a3], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) W[((e * p1 + b1) * M2 + a2) * M3 + a3] = acc[e];
    }
    __syncthreads();
    for (int s = lane; s < M1 * M2 * M3; s += tpe) {
      const int r = qdiv(s, rM3), a3 = s - r * M3, a1 = qdiv(r, rM2), a2 = r - a1 * M2;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int b1 = 0; b1 < p1; ++b1) {
        const T av = A[a1 + M1 * b1];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(av, W[((e * p1 + b1) * M2 + a2) * M3 + a3], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) y[e * nq + (M2 * a1 + a2) * M3 + a3] = acc[e];
    }
    __syncthreads();
  }
}

// x (NC x np) = V^T y (NC x nq); warped_product_2d.jl:61-89 / warped_product_3d.jl:94-136
template <typename T, int D, int NC>
__device__ void vdm_tmul(const DevOps &op, const T *y, T *x, T *Z, T *W, int lane, int tpe) {
  const int np = op.np, nq = op.nq;
  if (!op.has_vdm) {
    for (int t = lane; t < NC * nq; t += tpe) x[t] = y[t];
    __syncthreads();
    return;
  }
  if (op.dense_v) {
    // V^T with the dense V: one column of V per output mode
    const T *V = OpVals<T>::Vd(op);
    for (int a = lane; a < np; a += tpe) {
      const T *col = V + (size_t)nq * a;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int i = 0; i < nq; ++i) {
        const T v = col[i];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(v, y[e * nq + i], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) x[e * np + a] = acc[e];
    }
    __syncthreads();
    return;
  }
  const T *A = OpVals<T>::A(op), *B = OpVals<T>::B(op);
  const int p1 = op.p1, M1 = op.M1, M2 = op.M2;
  const float rM2 = qrcp(M2), rM3 = qrcp(op.M3 > 0 ? op.M3 : 1);
  if constexpr (D == 2) {
    for (int s = lane; s < p1 * M2; s += tpe) {
      const int b1 = qdiv(s, rM2), a2 = s - b1 * M2;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int a1 = 0; a1 < M1; ++a1) {
        const T av = A[a1 + M1 * b1];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(av, y[e * nq + M2 * a1 + a2], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) Z[(e * p1 + b1) * M2 + a2] = acc[e];
    }
    __syncthreads();
    for (int l = lane; l < np; l += tpe) {
      const int b1 = op.modes[l] & 0xff, b2 = (op.modes[l] >> 8) & 0xff;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int a2 = 0; a2 < M2; ++a2) {
        const T bv = B[a2 + M2 * (b1 + p1 * b2)];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(bv, Z[(e * p1 + b1) * M2 + a2], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) x[e * np + l] = acc[e];
    }
    __syncthreads();
  } else {
    const T *C = OpVals<T>::C(op);
    const int M3 = op.M3, nb12 = op.nb12;
    for (int s = lane; s < p1 * M2 * M3; s += tpe) {
      const int r = qdiv(s, rM3), a3 = s - r * M3, b1 = qdiv(r, rM2), a2 = r - b1 * M2;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int a1 = 0; a1 < M1; ++a1) {
        const T av = A[a1 + M1 * b1];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(av, y[e * nq + (M2 * a1 + a2) * M3 + a3], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) W[((e * p1 + b1) * M2 + a2) * M3 + a3] = acc[e];
    }
    __syncthreads();
    for (int s = lane; s < nb12 * M3; s += tpe) {
      const int q = qdiv(s, rM3), a3 = s - q * M3;
      const int b1 = op.b12[q] & 0xff, b2 = op.b12[q] >> 8;
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int a2 = 0; a2 < M2; ++a2) {
        const T bv = B[a2 + M2 * (b1 + p1 * b2)];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(bv, W[((e * p1 + b1) * M2 + a2) * M3 + a3], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) Z[(e * nb12 + q) * M3 + a3] = acc[e];
    }
    __syncthreads();
    for (int l = lane; l < np; l += tpe) {
      const int b1 = op.modes[l] & 0xff, b2 = (op.modes[l] >> 8) & 0xff, b3 = (op.modes[l] >> 16) & 0xff;
      const int q = op.b12_index[b1 + p1 * b2];
      T acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0;
      for (int a3 = 0; a3 < M3; ++a3) {
        const T cv = C[a3 + M3 * (b1 + p1 * (b2 + p1 * b3))];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(cv, Z[(e * nb12 + q) * M3 + a3], acc[e]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) x[e * np + l] = acc[e];
    }
    __syncthreads();
  }
}

// y (NC x rows) = M x (NC x cols) for a CSR matrix
template <typename T, int NC>
__device__ void csr_mul(int rows, int cols, const int *ptr, const int *idx, const T *val,
                        const T *x, T *y, int lane, int tpe) {
  for (int r = lane; r < rows; r += tpe) {
    T acc[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) acc[e] = 0;
    for (int q = ptr[r]; q < ptr[r + 1]; ++q) {
      const T v = val[q];
      const int c = idx[q];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] += v * x[e * cols + c];
    }
#pragma unroll
    for (int e = 0; e < NC; ++e) y[e * rows + r] = acc[e];
  }
}

// (R^T f)[e][i] for every volume node i (R^T rows in CSR, values Rtval in
// the form's scalar type), handed to sink(e * nq + i, value)
template <typename T, int NC, typename Sink>
__device__ __forceinline__ void rt_apply(const DevOps &op, const T *Rtval, const T *f, int lane,
                                         int tpe, Sink sink) {
  const int nq = op.nq, nf = op.nf;
  for (int i = lane; i < nq; i += tpe) {
    T acc[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) acc[e] = 0;
    for (int q = op.Rt_ptr[i]; q < op.Rt_ptr[i + 1]; ++q) {
      const T v = Rtval[q];
      const int c = op.Rt_idx[q];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = fma(v, f[e * nf + c], acc[e]);
    }
#pragma unroll
    for (int e = 0; e < NC; ++e) sink(e * nq + i, acc[e]);
  }
}

// WeightAdjustedSolver (M^-1 = I): x <- V^T diag(JinvW) V x;
// DiagonalSolver: x <- WJinv .* x (mass_matrix.jl:177-196)
// With Ak (the element's V' diag(J^-1 W) V, built once by mass_operator_kernel)
// the weight-adjusted solve is one dense product.  FP64 (issue-bound on the
// FP64 pipe): Ak column-major, one thread per (component, row), so N_c n_p
// threads share the FMAs where one thread per row would leave most of a team
// idle, and each column is one coalesced load.  FP32 (latency-bound): Ak
// row-major, one thread per row with N_c independent chains, which measured
// 5 % faster than both the FP64 scheme and column-major rows.
template <typename T, int D, int NC>
__device__ void mass_solve(const DevOps &op, const T *JinvW, const T *WJinv, int wa, T *x, T *Y,
                           T *Z, T *W, int lane, int tpe, const T *Ak = nullptr) {
  if (wa && Ak) {
    const int np = op.np;
    if constexpr (sizeof(T) == 8) {
      for (int t = lane; t < NC * np; t += tpe) {
        const int e = t / np, a = t - e * np;
        const T *xe = x + e * np;
        T acc = 0;
        for (int b = 0; b < np; ++b) acc = fma(Ak[(size_t)b * np + a], xe[b], acc);
        Y[t] = acc;
      }
    } else {
      // one row per S consecutive lanes (S = 1, 2 or 4, as many as the team
      // has threads for), each lane summing every S-th column, the partial
      // sums combined by shuffles in a fixed order; the team's warps run
      // the same number of rounds, so every shuffle sees its whole warp
      const int S = tpe >= 4 * np ? 4 : (tpe >= 2 * np ? 2 : 1);
      const int rounds = (np * S + tpe - 1) / tpe;
      for (int rd = 0; rd < rounds; ++rd) {
        const int t = rd * tpe + lane, a = t / S, sub = t - a * S;
        const bool act = a < np;
        const T *row = Ak + (size_t)(act ? a : 0) * np;
        T acc[NC];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = 0;
        if (act)
          for (int b = sub; b < np; b += S) {
            const T v = row[b];
#pragma unroll
            for (int e = 0; e < NC; ++e) acc[e] = fma(v, x[e * np + b], acc[e]);
          }
        for (int o = 1; o < S; o <<= 1)
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] += __shfl_xor_sync(0xffffffffu, acc[e], o);
        if (act && sub == 0)
#pragma unroll
          for (int e = 0; e < NC; ++e) Y[e * np + a] = acc[e];
      }
    }
    __syncthreads();
    for (int t = lane; t < NC * np; t += tpe) x[t] = Y[t];
    __syncthreads();
    return;
  }
  if (!wa) {
    for (int l = lane; l < op.np; l += tpe) {
      const T w = WJinv[l];
#pragma unroll
      for (int e = 0; e < NC; ++e) x[e * op.np + l] *= w;
    }
    __syncthreads();
    return;
  }
  vdm_mul<T, D, NC>(op, x, Y, Z, W, lane, tpe);
  for (int i = lane; i < op.nq; i += tpe) {
    const T w = JinvW[i];
#pragma unroll
    for (int e = 0; e < NC; ++e) Y[e * op.nq + i] *= w;
  }
  __syncthreads();
  vdm_tmul<T, D, NC>(op, Y, x, Z, W, lane, tpe);
}

// In-place Cholesky factorisation of the SPD n x n matrix M (row-major,
// lower triangle; the factor overwrites it) and solve of M y = b for nrhs
// right-hand sides Y[r][n], by the threads of one element team.  Sets *bad
// (shared) when a pivot is not positive.
__device__ __forceinline__ void team_cholesky_solve(double *M, int n, double *Y, int nrhs, int lane,
                                                    int tpe, int *bad) {
  for (int j = 0; j < n; ++j) {
    if (lane == 0) {
      double d = M[j * n + j];
      for (int q = 0; q < j; ++q) d = fma(-M[j * n + q], M[j * n + q], d);
      if (!(d > 0.0)) { *bad = 1; d = 1.0; }
      M[j * n + j] = sqrt(d);
    }
    __syncthreads();
    const double ljj = M[j * n + j];
    for (int i = j + 1 + lane; i < n; i += tpe) {
      double s = M[i * n + j];
      for (int q = 0; q < j; ++q) s = fma(-M[i * n + q], M[j * n + q], s);
      M[i * n + j] = s / ljj;
    }
    __syncthreads();
  }
  for (int e = lane; e < nrhs; e += tpe) {
    double *y = Y + (size_t)e * n;
    for (int r = 0; r < n; ++r) {
      double s = y[r];
      for (int q = 0; q < r; ++q) s = fma(-M[r * n + q], y[q], s);
      y[r] = s / M[r * n + r];
    }
    for (int r = n - 1; r >= 0; --r) {
      double s = y[r];
      for (int q = r + 1; q < n; ++q) s = fma(-M[q * n + r], y[q], s);
      y[r] = s / M[r * n + r];
    }
  }
  __syncthreads();
}

// Store one nodal state value: FP64 form -> the double scratch; mixed form ->
// the float scratch as a perturbation from the reference state.
template <int NC>
__device__ __forceinline__ void store_state(const KernelArgs &ka, double *d, float *f, size_t idx,
                                            int e, double v) {
  if (ka.mixed) {
    double ref = (e == 0) ? ka.ph.rho_ref : ((e == NC - 1) ? ka.ph.E_ref : 0.0);
    f[idx] = (float)(v - ref);
  } else {
    d[idx] = v;
  }
}


}  // namespace sse
