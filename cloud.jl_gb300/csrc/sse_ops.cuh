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

// y (NC x nq) = V x (NC x np); warped_product_2d.jl:31-55 / _3d.jl:47-84
template <typename T, int D, int NC>
__device__ void vdm_mul(const DevOps &op, const T *x, T *y, T *Z, T *W, int lane, int tpe) {
  if (!op.has_vdm) {
    for (int t = lane; t < NC * op.nq; t += tpe) y[t] = x[t];
    __syncthreads();
    return;
  }
  if (op.dense_v) {
    // dense V (multidimensional.jl:1-41): one row of V per output node
    const T *V = OpVals<T>::Vd(op);
    const int nq = op.nq, np = op.np;
    for (int t = lane; t < NC * nq; t += tpe) {
      const int i = t % nq, e = t / nq;
      T acc = 0;
      for (int a = 0; a < np; ++a) acc = fma(V[i + (size_t)nq * a], x[e * np + a], acc);
      y[t] = acc;
    }
    __syncthreads();
    return;
  }
  const T *A = OpVals<T>::A(op), *B = OpVals<T>::B(op);
  const int p1 = op.p1, M1 = op.M1, M2 = op.M2;
  if constexpr (D == 2) {
    // Z[e][b1][a2] = sum_b2 B[a2,b1,b2] x[sigma(b1,b2)]
    for (int t = lane; t < NC * p1 * M2; t += tpe) {
      int a2 = t % M2, r = t / M2, b1 = r % p1, e = r / p1;
      T acc = 0;
      for (int b2 = 0; b2 < p1 - b1; ++b2) {
        int l = modes_index2(op, b1, b2);
        acc = fma(B[a2 + M2 * (b1 + p1 * b2)], x[e * op.np + l], acc);
      }
      Z[(e * p1 + b1) * M2 + a2] = acc;
    }
    __syncthreads();
    for (int t = lane; t < NC * M1 * M2; t += tpe) {
      int a2 = t % M2, r = t / M2, a1 = r % M1, e = r / M1;
      T acc = 0;
      for (int b1 = 0; b1 < p1; ++b1) acc = fma(A[a1 + M1 * b1], Z[(e * p1 + b1) * M2 + a2], acc);
      y[e * op.nq + M2 * a1 + a2] = acc;
    }
    __syncthreads();
  } else {
    const T *C = OpVals<T>::C(op);
    const int M3 = op.M3, nb12 = op.nb12;
    for (int t = lane; t < NC * nb12 * M3; t += tpe) {
      int a3 = t % M3, r = t / M3, q = r % nb12, e = r / nb12;
      int b1 = op.b12[q] & 0xff, b2 = op.b12[q] >> 8;
      T acc = 0;
      for (int b3 = 0; b3 < p1 - b1 - b2; ++b3) {
        int l = modes_index3(op, b1, b2, b3);
        acc = fma(C[a3 + M3 * (b1 + p1 * (b2 + p1 * b3))], x[e * op.np + l], acc);
      }
      Z[(e * nb12 + q) * M3 + a3] = acc;
    }
    __syncthreads();
    for (int t = lane; t < NC * p1 * M2 * M3; t += tpe) {
      int a3 = t % M3, r = t / M3, a2 = r % M2, r2 = r / M2, b1 = r2 % p1, e = r2 / p1;
      T acc = 0;
      for (int b2 = 0; b2 < p1 - b1; ++b2) {
        int q = op.b12_index[b1 + p1 * b2];
        acc = fma(B[a2 + M2 * (b1 + p1 * b2)], Z[(e * nb12 + q) * M3 + a3], acc);
      }
      W[((e * p1 + b1) * M2 + a2) * M3 + a3] = acc;
    }
    __syncthreads();
    for (int t = lane; t < NC * M1 * M2 * M3; t += tpe) {
      int a3 = t % M3, r = t / M3, a2 = r % M2, r2 = r / M2, a1 = r2 % M1, e = r2 / M1;
      T acc = 0;
      for (int b1 = 0; b1 < p1; ++b1)
        acc = fma(A[a1 + M1 * b1], W[((e * p1 + b1) * M2 + a2) * M3 + a3], acc);
      y[e * op.nq + (M2 * a1 + a2) * M3 + a3] = acc;
    }
    __syncthreads();
  }
}

// x (NC x np) = V^T y (NC x nq); warped_product_2d.jl:61-89 / _3d.jl:94-136
template <typename T, int D, int NC>
__device__ void vdm_tmul(const DevOps &op, const T *y, T *x, T *Z, T *W, int lane, int tpe) {
  if (!op.has_vdm) {
    for (int t = lane; t < NC * op.nq; t += tpe) x[t] = y[t];
    __syncthreads();
    return;
  }
  if (op.dense_v) {
    // V^T with the dense V: one column of V per output mode
    const T *V = OpVals<T>::Vd(op);
    const int nq = op.nq, np = op.np;
    for (int t = lane; t < NC * np; t += tpe) {
      const int a = t % np, e = t / np;
      const T *col = V + (size_t)nq * a;
      T acc = 0;
      for (int i = 0; i < nq; ++i) acc = fma(col[i], y[e * nq + i], acc);
      x[t] = acc;
    }
    __syncthreads();
    return;
  }
  const T *A = OpVals<T>::A(op), *B = OpVals<T>::B(op);
  const int p1 = op.p1, M1 = op.M1, M2 = op.M2;
  if constexpr (D == 2) {
    for (int t = lane; t < NC * p1 * M2; t += tpe) {
      int a2 = t % M2, r = t / M2, b1 = r % p1, e = r / p1;
      T acc = 0;
      for (int a1 = 0; a1 < M1; ++a1) acc = fma(A[a1 + M1 * b1], y[e * op.nq + M2 * a1 + a2], acc);
      Z[(e * p1 + b1) * M2 + a2] = acc;
    }
    __syncthreads();
    for (int t = lane; t < NC * op.np; t += tpe) {
      int l = t % op.np, e = t / op.np;
      int b1 = op.modes[l] & 0xff, b2 = (op.modes[l] >> 8) & 0xff;
      T acc = 0;
      for (int a2 = 0; a2 < M2; ++a2) acc = fma(B[a2 + M2 * (b1 + p1 * b2)], Z[(e * p1 + b1) * M2 + a2], acc);
      x[e * op.np + l] = acc;
    }
    __syncthreads();
  } else {
    const T *C = OpVals<T>::C(op);
    const int M3 = op.M3, nb12 = op.nb12;
    for (int t = lane; t < NC * p1 * M2 * M3; t += tpe) {
      int a3 = t % M3, r = t / M3, a2 = r % M2, r2 = r / M2, b1 = r2 % p1, e = r2 / p1;
      T acc = 0;
      for (int a1 = 0; a1 < M1; ++a1)
        acc = fma(A[a1 + M1 * b1], y[e * op.nq + (M2 * a1 + a2) * M3 + a3], acc);
      W[((e * p1 + b1) * M2 + a2) * M3 + a3] = acc;
    }
    __syncthreads();
    for (int t = lane; t < NC * nb12 * M3; t += tpe) {
      int a3 = t % M3, r = t / M3, q = r % nb12, e = r / nb12;
      int b1 = op.b12[q] & 0xff, b2 = op.b12[q] >> 8;
      T acc = 0;
      for (int a2 = 0; a2 < M2; ++a2)
        acc = fma(B[a2 + M2 * (b1 + p1 * b2)], W[((e * p1 + b1) * M2 + a2) * M3 + a3], acc);
      Z[(e * nb12 + q) * M3 + a3] = acc;
    }
    __syncthreads();
    for (int t = lane; t < NC * op.np; t += tpe) {
      int l = t % op.np, e = t / op.np;
      int b1 = op.modes[l] & 0xff, b2 = (op.modes[l] >> 8) & 0xff, b3 = (op.modes[l] >> 16) & 0xff;
      int q = op.b12_index[b1 + p1 * b2];
      T acc = 0;
      for (int a3 = 0; a3 < M3; ++a3)
        acc = fma(C[a3 + M3 * (b1 + p1 * (b2 + p1 * b3))], Z[(e * nb12 + q) * M3 + a3], acc);
      x[e * op.np + l] = acc;
    }
    __syncthreads();
  }
}

// y (NC x rows) = M x (NC x cols) for a CSR matrix
template <typename T, int NC>
__device__ void csr_mul(int rows, int cols, const int *ptr, const int *idx, const T *val,
                        const T *x, T *y, int lane, int tpe) {
  for (int t = lane; t < NC * rows; t += tpe) {
    int r = t % rows, e = t / rows;
    T acc = 0;
    for (int q = ptr[r]; q < ptr[r + 1]; ++q) acc += val[q] * x[e * cols + idx[q]];
    y[e * rows + r] = acc;
  }
}

// WeightAdjustedSolver (M^-1 = I): x <- V^T diag(JinvW) V x;
// DiagonalSolver: x <- WJinv .* x (mass_matrix.jl:177-196)
template <typename T, int D, int NC>
__device__ void mass_solve(const DevOps &op, const T *JinvW, const T *WJinv, int wa, T *x, T *Y,
                           T *Z, T *W, int lane, int tpe) {
  if (!wa) {
    for (int t = lane; t < NC * op.np; t += tpe) x[t] *= WJinv[t % op.np];
    __syncthreads();
    return;
  }
  vdm_mul<T, D, NC>(op, x, Y, Z, W, lane, tpe);
  for (int t = lane; t < NC * op.nq; t += tpe) Y[t] *= JinvW[t % op.nq];
  __syncthreads();
  vdm_tmul<T, D, NC>(op, Y, x, Z, W, lane, tpe);
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
