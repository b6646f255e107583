// sse_project.cu -- L2 projection of initial data onto the modal basis, FP64.
//
// project_function (src/Solvers/Solvers.jl:396-418): per element the mass
// matrix M = VDM' diag(W J) VDM is formed, factorised by Cholesky and solved
// against VDM' (W J u_q), all in one CTA: the weights, nodal data, mass
// matrix, factor and right-hand sides live in shared memory; VDM is read
// through L1/L2 by every CTA.
#include <cmath>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sse_gb300.h"
#include "sse_kernels.cuh"

namespace sse {
namespace {

struct ProjArgs {
  int np, nq, nc;
  const double *V, *W, *J, *uq;
  double *u0;
  int *flag;  // set when a mass matrix is not positive definite
};

// Shared memory: WJ[nq], U[nc][nq] (then W J u), M[np][np] (lower triangle,
// overwritten by the Cholesky factor), Y[nc][np].
__global__ void __launch_bounds__(128) project_function_kernel(ProjArgs a) {
  extern __shared__ double sm[];
  const int64_t k = blockIdx.x;
  const int np = a.np, nq = a.nq, nc = a.nc;
  double *WJ = sm, *U = WJ + nq, *M = U + (size_t)nc * nq, *Y = M + (size_t)np * np;
  for (int i = threadIdx.x; i < nq; i += blockDim.x) WJ[i] = a.W[i] * a.J[(size_t)nq * k + i];
  for (int t = threadIdx.x; t < nc * nq; t += blockDim.x) U[t] = a.uq[(size_t)nc * nq * k + t];
  __syncthreads();
  // lmul!(WJ, u_q): U <- WJ .* U
  for (int t = threadIdx.x; t < nc * nq; t += blockDim.x) U[t] *= WJ[t % nq];
  // M[r][c] (r >= c) = sum_i VDM[i, r] WJ[i] VDM[i, c]
  const int ntri = np * (np + 1) / 2;
  for (int t = threadIdx.x; t < ntri; t += blockDim.x) {
    // t -> (r, c) with c <= r, rows in order
    int r = (int)((sqrt(8.0 * t + 1.0) - 1.0) * 0.5);
    while (r * (r + 1) / 2 > t) --r;
    while ((r + 1) * (r + 2) / 2 <= t) ++r;
    const int c = t - r * (r + 1) / 2;
    const double *vr = a.V + (size_t)nq * r, *vc = a.V + (size_t)nq * c;
    double acc = 0.0;
    for (int i = 0; i < nq; ++i) acc = fma(__ldg(vr + i) * WJ[i], __ldg(vc + i), acc);
    M[r * np + c] = acc;
  }
  __syncthreads();
  // right-hand sides Y[e][r] = sum_i VDM[i, r] (WJ u_q)[e][i]
  for (int t = threadIdx.x; t < nc * np; t += blockDim.x) {
    const int e = t / np, r = t - e * np;
    const double *vr = a.V + (size_t)nq * r;
    double acc = 0.0;
    for (int i = 0; i < nq; ++i) acc = fma(__ldg(vr + i), U[e * nq + i], acc);
    Y[t] = acc;
  }
  // Cholesky M = L L' by columns (L overwrites the lower triangle)
  __shared__ int bad;
  if (threadIdx.x == 0) bad = 0;
  __syncthreads();
  for (int j = 0; j < np; ++j) {
    if (threadIdx.x == 0) {
      double d = M[j * np + j];
      for (int q = 0; q < j; ++q) d = fma(-M[j * np + q], M[j * np + q], d);
      if (!(d > 0.0)) { bad = 1; d = 1.0; }
      M[j * np + j] = sqrt(d);
    }
    __syncthreads();
    const double ljj = M[j * np + j];
    for (int i = j + 1 + threadIdx.x; i < np; i += blockDim.x) {
      double s = M[i * np + j];
      for (int q = 0; q < j; ++q) s = fma(-M[i * np + q], M[j * np + q], s);
      M[i * np + j] = s / ljj;
    }
    __syncthreads();
  }
  // L z = y, L' x = z, one right-hand side per thread
  for (int e = threadIdx.x; e < nc; e += blockDim.x) {
    double *y = Y + (size_t)e * np;
    for (int r = 0; r < np; ++r) {
      double s = y[r];
      for (int q = 0; q < r; ++q) s = fma(-M[r * np + q], y[q], s);
      y[r] = s / M[r * np + r];
    }
    for (int r = np - 1; r >= 0; --r) {
      double s = y[r];
      for (int q = r + 1; q < np; ++q) s = fma(-M[q * np + r], y[q], s);
      y[r] = s / M[r * np + r];
    }
  }
  __syncthreads();
  for (int t = threadIdx.x; t < nc * np; t += blockDim.x) a.u0[(size_t)nc * np * k + t] = Y[t];
  if (threadIdx.x == 0 && bad) atomicExch(a.flag, 1);
}

struct Buffers {
  std::vector<void *> ptrs;
  ~Buffers() {
    for (void *p : ptrs) cudaFree(p);
  }
  cudaError_t alloc(size_t bytes, void **out) {
    *out = nullptr;
    cudaError_t e = cudaMalloc(out, bytes > 0 ? bytes : 8);
    if (e == cudaSuccess) ptrs.push_back(*out);
    return e;
  }
};

}  // namespace

int project_function_run(int np, int nq, int nc, int64_t ne, const double *V, const double *W,
                         const double *J, const double *uq, double *u0, int memory, std::string *err) {
  auto bad = [&](const char *msg) {
    *err = msg;
    return (int)SSE_ERR_INVALID_ARGUMENT;
  };
  if (np <= 0 || nq <= 0 || nc <= 0 || nc > 8 || ne <= 0 || ne > 0x7fffffff) return bad("bad sizes");
  if (np > nq) return bad("n_p must not exceed n_q");
  if (!V || !W || !J || !uq || !u0) return bad("null array");
  if (memory != SSE_HOST && memory != SSE_DEVICE) return bad("memory must be SSE_HOST or SSE_DEVICE");
  const size_t smem = ((size_t)nq + (size_t)nc * nq + (size_t)np * np + (size_t)nc * np) * sizeof(double);
  int dev = 0, optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > (size_t)optin) {
    *err = "element too large for one CTA's shared memory";
    return SSE_ERR_UNSUPPORTED;
  }
  Buffers buf;
  auto cuda = [&](cudaError_t e, const char *where) {
    *err = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? (int)SSE_ERR_OUT_OF_MEMORY : (int)SSE_ERR_CUDA;
  };
  cudaError_t e;
  void *p;
  ProjArgs a{};
  a.np = np;
  a.nq = nq;
  a.nc = nc;
  if ((e = buf.alloc(((size_t)nq * np + nq) * sizeof(double), &p)) != cudaSuccess) return cuda(e, "allocate");
  a.V = (const double *)p;
  a.W = a.V + (size_t)nq * np;
  if ((e = cudaMemcpy(p, V, (size_t)nq * np * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
      (e = cudaMemcpy((double *)p + (size_t)nq * np, W, nq * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
    return cuda(e, "upload VDM, W");
  if ((e = buf.alloc(sizeof(int), &p)) != cudaSuccess) return cuda(e, "allocate");
  a.flag = (int *)p;
  if ((e = cudaMemset(a.flag, 0, sizeof(int))) != cudaSuccess) return cuda(e, "memset");
  const size_t n_j = (size_t)nq * ne, n_u = (size_t)nq * nc * ne, n_o = (size_t)np * nc * ne;
  if (memory == SSE_DEVICE) {
    a.J = J;
    a.uq = uq;
    a.u0 = u0;
  } else {
    if ((e = buf.alloc((n_j + n_u + n_o) * sizeof(double), &p)) != cudaSuccess) return cuda(e, "allocate");
    double *d = (double *)p;
    if ((e = cudaMemcpy(d, J, n_j * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess ||
        (e = cudaMemcpy(d + n_j, uq, n_u * sizeof(double), cudaMemcpyHostToDevice)) != cudaSuccess)
      return cuda(e, "upload J_q, u_q");
    a.J = d;
    a.uq = d + n_j;
    a.u0 = d + n_j + n_u;
  }
  cudaFuncSetAttribute(project_function_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  project_function_kernel<<<(unsigned)ne, 128, smem>>>(a);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda(e, "projection kernel launch");
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda(e, "projection kernel");
  int flag = 0;
  if ((e = cudaMemcpy(&flag, a.flag, sizeof(int), cudaMemcpyDeviceToHost)) != cudaSuccess) return cuda(e, "flag");
  if (memory == SSE_HOST &&
      (e = cudaMemcpy(u0, a.u0, n_o * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess)
    return cuda(e, "copy u0 to the host");
  if (flag) {
    *err = "a mass matrix is not positive definite";
    return SSE_ERR_NONPHYSICAL;
  }
  return SSE_OK;
}

}  // namespace sse
