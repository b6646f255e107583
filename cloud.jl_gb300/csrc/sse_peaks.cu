// sse_peaks.cu -- measured FP64 / FP32 CUDA-core FMA throughput of the
// current device, the denominators of the residual kernels' roofline
// (the FP64 form is bound by the FP64 pipe, not by HBM or tensor cores).
#include <cuda_runtime.h>

#include "../../include/sse_gb300.h"

namespace {

constexpr int kChains = 8;

template <typename T>
__global__ void fma_chains(T *out, int iters, T a, T b) {
  T x[kChains];
#pragma unroll
  for (int c = 0; c < kChains; ++c) x[c] = (T)(threadIdx.x + c);
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int c = 0; c < kChains; ++c) x[c] = fma(x[c], a, b);
  }
  T s = 0;
#pragma unroll
  for (int c = 0; c < kChains; ++c) s += x[c];
  if (s == (T)-1.2345) out[0] = s;  // keeps the chains live; never true for these inputs
}

template <typename T>
double measure(int iters, T *scratch) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const int threads = 256, blocks = sms * 8;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  fma_chains<T><<<blocks, threads>>>(scratch, iters / 10, (T)0.999999, (T)1e-7);  // warm-up
  cudaEventRecord(e0);
  fma_chains<T><<<blocks, threads>>>(scratch, iters, (T)0.999999, (T)1e-7);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  double flops = 2.0 * kChains * (double)iters * threads * blocks;
  return flops / (ms * 1e-3) / 1e12;
}

}  // namespace

extern "C" int32_t sse_measure_fma_peaks(double *out) {
  if (!out) return SSE_ERR_INVALID_ARGUMENT;
  void *scratch = nullptr;
  if (cudaMalloc(&scratch, 64) != cudaSuccess) return SSE_ERR_CUDA;
  out[0] = measure<double>(1 << 14, (double *)scratch);
  out[1] = measure<float>(1 << 16, (float *)scratch);
  cudaError_t e = cudaGetLastError();
  cudaFree(scratch);
  return e == cudaSuccess ? SSE_OK : SSE_ERR_CUDA;
}
