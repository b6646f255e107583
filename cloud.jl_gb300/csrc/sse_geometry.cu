// sse_geometry.cu -- GeometricFactors on the device, FP64.
//
// Restates, one CTA per element, the constructors
//   GeometricFactors(mesh, reference_element, ExactMetrics())
//       src/SpatialDiscretizations/mesh.jl:229-282
//   GeometricFactors(mesh::MeshData{2}, ..., ConservativeCurlMetrics())
//       mesh.jl:284-339 (StartUpDG's 2-D geometric_factors at the mapping nodes)
//   GeometricFactors(mesh::MeshData{3}, ::RefElemData{3, Tet}, ConservativeCurlMetrics())
//       mesh.jl:410-506 (metric terms as curls of degree N+1 interpolants)
// and project_jacobian! (SpatialDiscretizations.jl:310-317).  The reference
// evaluates each step as a matrix product over all elements; here an
// element's coordinates, derivatives and metric terms stay in shared memory
// and only the GeometricFactors fields are written to HBM.  The reference
// matrices (a few hundred KB at most) are read through L1/L2 by every CTA;
// each load feeds 3 to 18 FMAs (the vectors sharing that matrix).
#include <cmath>
#include <string>
#include <utility>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/sse_gb300.h"
#include "sse_kernels.cuh"

namespace sse {
namespace {

struct MetricArgs {
  int n_map, n_q, n_f, num_faces, npf, n1, project;
  const double *Dr[3], *Vq, *Vf, *nrstJ[3];
  const double *N1, *D1[3], *Vq1, *Vf1, *P;
  const double *xyz[3];
  double *J_q, *Lambda_q, *J_f, *nJf, *nJq;
};

template <int NA>
struct Mats {
  const double *p[NA];
};

// y_v[i] = sum_j A_a[i, j] x_v[j] for the NA matrices A_a (column-major,
// m x n) and the NX vectors x_v in shared memory (stride xs); the result for
// matrix a and vector v goes to y[(a * NX + v) * ys + i].  Rows are strided
// over the CTA's threads.
template <int NA, int NX>
__device__ __forceinline__ void matvecs(Mats<NA> A, int m, int n, const double *x,
                                        int xs, double *y, int ys) {
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    double acc[NA][NX];
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int v = 0; v < NX; ++v) acc[a][v] = 0.0;
    for (int j = 0; j < n; ++j) {
      double xv[NX];
#pragma unroll
      for (int v = 0; v < NX; ++v) xv[v] = x[v * xs + j];
#pragma unroll
      for (int a = 0; a < NA; ++a) {
        const double aij = __ldg(A.p[a] + i + (size_t)j * m);
#pragma unroll
        for (int v = 0; v < NX; ++v) acc[a][v] = fma(aij, xv[v], acc[a][v]);
      }
    }
#pragma unroll
    for (int a = 0; a < NA; ++a)
#pragma unroll
      for (int v = 0; v < NX; ++v) y[(a * NX + v) * ys + i] = acc[a][v];
  }
}

// Row i of A (m x n, column-major) applied to NV vectors in shared memory.
template <int NV>
__device__ __forceinline__ void row_apply(const double *__restrict__ A, int m, int n, int i,
                                          const double *x, int xs, double *acc) {
#pragma unroll
  for (int v = 0; v < NV; ++v) acc[v] = 0.0;
  for (int j = 0; j < n; ++j) {
    const double aij = __ldg(A + i + (size_t)j * m);
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = fma(aij, x[v * xs + j], acc[v]);
  }
}

// metrics(dxdr) of mesh.jl:217-227: J = det(A) and Λ = J inv(A) = adj(A),
// A[m][n] = ∂x_m/∂r_n.
template <int D>
__device__ __forceinline__ double adjugate(const double (&a)[D][D], double (&adj)[D][D]) {
  if constexpr (D == 2) {
    adj[0][0] = a[1][1];
    adj[0][1] = -a[0][1];
    adj[1][0] = -a[1][0];
    adj[1][1] = a[0][0];
    return a[0][0] * a[1][1] - a[0][1] * a[1][0];
  } else {
    adj[0][0] = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    adj[0][1] = a[0][2] * a[2][1] - a[0][1] * a[2][2];
    adj[0][2] = a[0][1] * a[1][2] - a[0][2] * a[1][1];
    adj[1][0] = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    adj[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
    adj[1][2] = a[0][2] * a[1][0] - a[0][0] * a[1][2];
    adj[2][0] = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    adj[2][1] = a[0][1] * a[2][0] - a[0][0] * a[2][1];
    adj[2][2] = a[0][0] * a[1][1] - a[0][1] * a[1][0];
    return a[0][0] * adj[0][0] + a[0][1] * adj[1][0] + a[0][2] * adj[2][0];
  }
}

// nJq[n, f, i, k] = sum_m Λ[i, m, n] nrstJ[m][npf f] (mesh.jl:262-269) from
// the node's metric terms L[m + D n].
template <int D>
__device__ __forceinline__ void write_nJq(const MetricArgs &g, int64_t k, int i, const double *L) {
  double *out = g.nJq + (size_t)D * g.num_faces * ((size_t)g.n_q * k + i);
  for (int f = 0; f < g.num_faces; ++f) {
    const int r = g.npf * f;
#pragma unroll
    for (int n = 0; n < D; ++n) {
      double acc = L[0 + D * n] * __ldg(g.nrstJ[0] + r);
#pragma unroll
      for (int m = 1; m < D; ++m) acc += L[m + D * n] * __ldg(g.nrstJ[m] + r);
      out[D * f + n] = acc;
    }
  }
}

// nJf[m, i, k] = sum_n Λ_f[i, n, m] nrstJ[n][i]; J_f = |nJf| (mesh.jl:272-279).
template <int D>
__device__ __forceinline__ void write_nJf(const MetricArgs &g, int64_t k, int i, const double *L) {
  double *out = g.nJf + (size_t)D * ((size_t)g.n_f * k + i);
  double s = 0.0;
#pragma unroll
  for (int m = 0; m < D; ++m) {
    double acc = L[0 + D * m] * __ldg(g.nrstJ[0] + i);
#pragma unroll
    for (int n = 1; n < D; ++n) acc += L[n + D * m] * __ldg(g.nrstJ[n] + i);
    out[m] = acc;
    s += acc * acc;
  }
  g.J_f[(size_t)g.n_f * k + i] = sqrt(s);
}

template <int D>
__device__ __forceinline__ void store_lambda(const MetricArgs &g, int64_t k, int i, const double *L) {
  double *out = g.Lambda_q + (size_t)D * D * g.n_q * k + i;
#pragma unroll
  for (int v = 0; v < D * D; ++v) out[(size_t)v * g.n_q] = L[v];
}

__device__ __forceinline__ void load_xyz(const MetricArgs &g, int64_t k, int D, double *X) {
  for (int t = threadIdx.x; t < D * g.n_map; t += blockDim.x) {
    const int c = t / g.n_map, i = t - c * g.n_map;
    X[t] = g.xyz[c][(size_t)g.n_map * k + i];
  }
}

// Exact metrics: derivatives of the degree-N mapping at the mapping nodes,
// interpolated to the quadrature / facet nodes, then metrics() per node.
// Shared memory: X[D][n_map], G[D*D][n_map], Jq[n_q] (projection only).
template <int D>
__global__ void __launch_bounds__(128) exact_metrics_kernel(MetricArgs g) {
  extern __shared__ double sm[];
  const int64_t k = blockIdx.x;
  double *X = sm;
  double *G = X + D * g.n_map;          // G[(a * D + c)] = D_a x_c
  double *Jq = G + D * D * g.n_map;
  load_xyz(g, k, D, X);
  Mats<D> Dm;
#pragma unroll
  for (int a = 0; a < D; ++a) Dm.p[a] = g.Dr[a];
  __syncthreads();
  matvecs<D, D>(Dm, g.n_map, g.n_map, X, g.n_map, G, g.n_map);
  __syncthreads();
  for (int i = threadIdx.x; i < g.n_q; i += blockDim.x) {
    double acc[D * D];
    row_apply<D * D>(g.Vq, g.n_q, g.n_map, i, G, g.n_map, acc);
    double a[D][D], adj[D][D];
#pragma unroll
    for (int m = 0; m < D; ++m)
#pragma unroll
      for (int n = 0; n < D; ++n) a[m][n] = acc[n * D + m];
    const double J = adjugate<D>(a, adj);
    double L[D * D];
#pragma unroll
    for (int m = 0; m < D; ++m)
#pragma unroll
      for (int n = 0; n < D; ++n) L[m + D * n] = adj[m][n];
    store_lambda<D>(g, k, i, L);
    write_nJq<D>(g, k, i, L);
    if (g.project) Jq[i] = J;
    else g.J_q[(size_t)g.n_q * k + i] = J;
  }
  for (int i = threadIdx.x; i < g.n_f; i += blockDim.x) {
    double acc[D * D];
    row_apply<D * D>(g.Vf, g.n_f, g.n_map, i, G, g.n_map, acc);
    double a[D][D], adj[D][D];
#pragma unroll
    for (int m = 0; m < D; ++m)
#pragma unroll
      for (int n = 0; n < D; ++n) a[m][n] = acc[n * D + m];
    adjugate<D>(a, adj);
    double L[D * D];
#pragma unroll
    for (int m = 0; m < D; ++m)
#pragma unroll
      for (int n = 0; n < D; ++n) L[m + D * n] = adj[m][n];
    write_nJf<D>(g, k, i, L);
  }
  if (g.project) {
    __syncthreads();
    for (int i = threadIdx.x; i < g.n_q; i += blockDim.x) {
      double acc[1];
      row_apply<1>(g.P, g.n_q, g.n_q, i, Jq, g.n_q, acc);
      g.J_q[(size_t)g.n_q * k + i] = acc[0];
    }
  }
}

// 2-D conservative-curl metrics (mesh.jl:284-339): rxJ = y_s, sxJ = -y_r,
// ryJ = -x_s, syJ = x_r, J = -x_s y_r + x_r y_s at the mapping nodes, then
// interpolated.  Shared memory: X[2][n_map], G[4][n_map], M[5][n_map].
__global__ void __launch_bounds__(128) curl_metrics_2d_kernel(MetricArgs g) {
  extern __shared__ double sm[];
  const int64_t k = blockIdx.x;
  const int nm = g.n_map;
  double *X = sm;
  double *G = X + 2 * nm;
  double *M = G + 4 * nm;   // M[m + 2 n] = Λ[m, n], M[4] = J
  load_xyz(g, k, 2, X);
  __syncthreads();
  matvecs<2, 2>(Mats<2>{{g.Dr[0], g.Dr[1]}}, nm, nm, X, nm, G, nm);
  __syncthreads();
  for (int i = threadIdx.x; i < nm; i += blockDim.x) {
    const double xr = G[0 * nm + i], yr = G[1 * nm + i];
    const double xs = G[2 * nm + i], ys = G[3 * nm + i];
    M[0 * nm + i] = ys;
    M[1 * nm + i] = -yr;
    M[2 * nm + i] = -xs;
    M[3 * nm + i] = xr;
    M[4 * nm + i] = -xs * yr + xr * ys;
  }
  __syncthreads();
  for (int i = threadIdx.x; i < g.n_q; i += blockDim.x) {
    double acc[5];
    row_apply<5>(g.Vq, g.n_q, nm, i, M, nm, acc);
    store_lambda<2>(g, k, i, acc);
    write_nJq<2>(g, k, i, acc);
    g.J_q[(size_t)g.n_q * k + i] = acc[4];
  }
  for (int i = threadIdx.x; i < g.n_f; i += blockDim.x) {
    double acc[4];
    row_apply<4>(g.Vf, g.n_f, nm, i, M, nm, acc);
    write_nJf<2>(g, k, i, acc);
  }
}

// 3-D conservative-curl metrics on the Tet (mesh.jl:410-506).  J from the
// degree-N mapping at its nodes (StartUpDG's geometric_factors), the metric
// terms as curls (Kopriva 2006) of degree N+1 interpolants,
//   (J ∇ξ_a)_n = -ê_n · ∇_ξ × (x_l ∇_ξ x_m),
// brought back through Vq * Nplus1_to_N.  Shared memory: X[3][n_map],
// G[9][n_map], Jm[n_map], X1[3][n1], G1[9][n1] (reused for the metric terms),
// F[9][n1].
__global__ void __launch_bounds__(128) curl_metrics_3d_kernel(MetricArgs g) {
  extern __shared__ double sm[];
  const int64_t k = blockIdx.x;
  const int nm = g.n_map, n1 = g.n1;
  double *X = sm;
  double *G = X + 3 * nm;     // G[a * 3 + c] = D_a x_c
  double *Jm = G + 9 * nm;
  double *X1 = Jm + nm;
  double *G1 = X1 + 3 * n1;   // D1_a x1_c, later the metric terms M[m + 3 n]
  double *F = G1 + 9 * n1;    // F[p * 3 + a]
  load_xyz(g, k, 3, X);
  __syncthreads();
  matvecs<3, 3>(Mats<3>{{g.Dr[0], g.Dr[1], g.Dr[2]}}, nm, nm, X, nm, G, nm);
  matvecs<1, 3>(Mats<1>{{g.N1}}, n1, nm, X, nm, X1, n1);
  __syncthreads();
  for (int i = threadIdx.x; i < nm; i += blockDim.x) {
    const double xr = G[0 * nm + i], yr = G[1 * nm + i], zr = G[2 * nm + i];
    const double xs = G[3 * nm + i], ys = G[4 * nm + i], zs = G[5 * nm + i];
    const double xt = G[6 * nm + i], yt = G[7 * nm + i], zt = G[8 * nm + i];
    Jm[i] = xr * (ys * zt - zs * yt) - yr * (xs * zt - zs * xt) + zr * (xs * yt - ys * xt);
  }
  matvecs<3, 3>(Mats<3>{{g.D1[0], g.D1[1], g.D1[2]}}, n1, n1, X1, n1, G1, n1);
  __syncthreads();
  for (int i = threadIdx.x; i < g.n_q; i += blockDim.x) {
    double acc[1];
    row_apply<1>(g.Vq, g.n_q, nm, i, Jm, nm, acc);
    g.J_q[(size_t)g.n_q * k + i] = acc[0];
  }
  // pairs (differentiated, multiplier): (y, z) -> n = x, (x, z) -> n = y
  // (negated), (y, x) -> n = z (negated)
  for (int i = threadIdx.x; i < n1; i += blockDim.x) {
    const int dc[3] = {1, 0, 1}, mc[3] = {2, 2, 0};
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int a = 0; a < 3; ++a) F[(p * 3 + a) * n1 + i] = G1[(a * 3 + dc[p]) * n1 + i] * X1[mc[p] * n1 + i];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < n1; i += blockDim.x) {
    // per pair: D_t F_s, D_s F_t, D_r F_t, D_t F_r, D_s F_r, D_r F_s
    double acc[3][6];
#pragma unroll
    for (int p = 0; p < 3; ++p)
#pragma unroll
      for (int q = 0; q < 6; ++q) acc[p][q] = 0.0;
    for (int j = 0; j < n1; ++j) {
      const size_t o = i + (size_t)j * n1;
      const double dr = __ldg(g.D1[0] + o), ds = __ldg(g.D1[1] + o), dt = __ldg(g.D1[2] + o);
#pragma unroll
      for (int p = 0; p < 3; ++p) {
        const double fr = F[(p * 3 + 0) * n1 + j], fs = F[(p * 3 + 1) * n1 + j],
                     ft = F[(p * 3 + 2) * n1 + j];
        acc[p][0] = fma(dt, fs, acc[p][0]);
        acc[p][1] = fma(ds, ft, acc[p][1]);
        acc[p][2] = fma(dr, ft, acc[p][2]);
        acc[p][3] = fma(dt, fr, acc[p][3]);
        acc[p][4] = fma(ds, fr, acc[p][4]);
        acc[p][5] = fma(dr, fs, acc[p][5]);
      }
    }
#pragma unroll
    for (int p = 0; p < 3; ++p) {
      const double c0 = acc[p][0] - acc[p][1];
      const double c1 = acc[p][2] - acc[p][3];
      const double c2 = acc[p][4] - acc[p][5];
      const double sgn = p == 0 ? 1.0 : -1.0;
      G1[(0 + 3 * p) * n1 + i] = sgn * c0;
      G1[(1 + 3 * p) * n1 + i] = sgn * c1;
      G1[(2 + 3 * p) * n1 + i] = sgn * c2;
    }
  }
  __syncthreads();
  for (int i = threadIdx.x; i < g.n_q; i += blockDim.x) {
    double L[9];
    row_apply<9>(g.Vq1, g.n_q, n1, i, G1, n1, L);
    store_lambda<3>(g, k, i, L);
    write_nJq<3>(g, k, i, L);
  }
  for (int i = threadIdx.x; i < g.n_f; i += blockDim.x) {
    double L[9];
    row_apply<9>(g.Vf1, g.n_f, n1, i, G1, n1, L);
    write_nJf<3>(g, k, i, L);
  }
}

struct DeviceBuffers {
  std::vector<void *> ptrs;
  ~DeviceBuffers() {
    for (void *p : ptrs) cudaFree(p);
  }
  cudaError_t alloc(size_t bytes, void **out) {
    *out = nullptr;
    cudaError_t e = cudaMalloc(out, bytes > 0 ? bytes : 8);
    if (e == cudaSuccess) ptrs.push_back(*out);
    return e;
  }
  cudaError_t upload(const double *host, size_t n, const double **dev) {
    void *p = nullptr;
    cudaError_t e = alloc(n * sizeof(double), &p);
    if (e != cudaSuccess) return e;
    *dev = (const double *)p;
    return cudaMemcpy(p, host, n * sizeof(double), cudaMemcpyHostToDevice);
  }
};

// The reference matrices packed into one host block and one device
// allocation: one copy per call instead of one per matrix.
struct OperatorPack {
  std::vector<double> host;
  std::vector<std::pair<const double **, size_t>> slots;  // (destination, offset)
  void add(const double *src, size_t n, const double **dst) {
    slots.push_back({dst, host.size()});
    host.insert(host.end(), src, src + n);
  }
  cudaError_t upload(DeviceBuffers &buf) {
    const double *dev = nullptr;
    cudaError_t e = buf.upload(host.data(), host.size(), &dev);
    if (e != cudaSuccess) return e;
    for (auto &s : slots) *s.first = dev + s.second;
    return cudaSuccess;
  }
};

}  // namespace

int geometric_factors_run(const sse_metric_operators *ops, int64_t n_e, const double *const *xyz,
                          const sse_geometric_factors_out *out, int memory, std::string *err) {
  auto bad = [&](const char *msg) {
    *err = msg;
    return (int)SSE_ERR_INVALID_ARGUMENT;
  };
  if (!ops || !xyz || !out) return bad("null operators, coordinates or outputs");
  const int d = ops->d;
  if (d != 2 && d != 3) return bad("d must be 2 or 3");
  if (ops->metrics != SSE_EXACT_METRICS && ops->metrics != SSE_CONSERVATIVE_CURL_METRICS)
    return bad("unknown metric type");
  if (memory != SSE_HOST && memory != SSE_DEVICE) return bad("memory must be SSE_HOST or SSE_DEVICE");
  if (n_e <= 0 || n_e > 0x7fffffff) return bad("n_e out of range");
  if (ops->n_map <= 0 || ops->n_q <= 0 || ops->n_f <= 0 || ops->num_faces <= 0 ||
      ops->n_f % ops->num_faces != 0)
    return bad("bad sizes (n_map, n_q, n_f, num_faces)");
  if (!ops->Vq || !ops->Vf) return bad("Vq and Vf are required");
  for (int m = 0; m < d; ++m) {
    if (!ops->Drst[m] || !ops->nrstJ[m] || !xyz[m]) return bad("Drst, nrstJ and xyz need d entries");
  }
  const bool curl3 = ops->metrics == SSE_CONSERVATIVE_CURL_METRICS && d == 3;
  if (curl3) {
    if (ops->n_curl <= 0 || !ops->N_to_Nplus1 || !ops->Vq_Nplus1 || !ops->Vf_Nplus1 ||
        !ops->Drst_Nplus1[0] || !ops->Drst_Nplus1[1] || !ops->Drst_Nplus1[2])
      return bad("3-D curl metrics need n_curl, N_to_Nplus1, Drst_Nplus1, Vq_Nplus1, Vf_Nplus1");
  }
  if (ops->project_jacobian && (ops->metrics != SSE_EXACT_METRICS || !ops->project))
    return bad("project_jacobian applies to exact metrics and needs the projection matrix");
  if (!out->J_q || !out->Lambda_q || !out->J_f || !out->nJf || !out->nJq)
    return bad("every GeometricFactors output is required");

  const int nm = ops->n_map, nq = ops->n_q, nf = ops->n_f, n1 = curl3 ? ops->n_curl : 0;
  size_t smem_doubles;
  if (ops->metrics == SSE_EXACT_METRICS)
    smem_doubles = (size_t)(d + d * d) * nm + (ops->project_jacobian ? nq : 0);
  else if (d == 2)
    smem_doubles = (size_t)11 * nm;
  else
    smem_doubles = (size_t)13 * nm + (size_t)21 * n1;
  const size_t smem = smem_doubles * sizeof(double);
  int dev = 0, max_optin = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&max_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
  if (smem > (size_t)max_optin) {
    *err = "element too large for one CTA's shared memory";
    return SSE_ERR_UNSUPPORTED;
  }

  DeviceBuffers buf;
  auto cuda = [&](cudaError_t e, const char *where) {
    *err = std::string(where) + ": " + cudaGetErrorString(e);
    return e == cudaErrorMemoryAllocation ? (int)SSE_ERR_OUT_OF_MEMORY : (int)SSE_ERR_CUDA;
  };
  cudaError_t e;
  MetricArgs g{};
  g.n_map = nm;
  g.n_q = nq;
  g.n_f = nf;
  g.num_faces = ops->num_faces;
  g.npf = nf / ops->num_faces;
  g.n1 = n1;
  g.project = ops->project_jacobian ? 1 : 0;
  OperatorPack pack;
  for (int m = 0; m < d; ++m) {
    pack.add(ops->Drst[m], (size_t)nm * nm, &g.Dr[m]);
    pack.add(ops->nrstJ[m], nf, &g.nrstJ[m]);
  }
  pack.add(ops->Vq, (size_t)nq * nm, &g.Vq);
  pack.add(ops->Vf, (size_t)nf * nm, &g.Vf);
  if (curl3) {
    pack.add(ops->N_to_Nplus1, (size_t)n1 * nm, &g.N1);
    for (int m = 0; m < 3; ++m) pack.add(ops->Drst_Nplus1[m], (size_t)n1 * n1, &g.D1[m]);
    pack.add(ops->Vq_Nplus1, (size_t)nq * n1, &g.Vq1);
    pack.add(ops->Vf_Nplus1, (size_t)nf * n1, &g.Vf1);
  }
  if (g.project) pack.add(ops->project, (size_t)nq * nq, &g.P);
  if ((e = pack.upload(buf)) != cudaSuccess) return cuda(e, "upload reference matrices");

  const size_t ne = (size_t)n_e;
  const size_t len[5] = {(size_t)nq * ne, (size_t)nq * d * d * ne, (size_t)nf * ne,
                         (size_t)d * nf * ne, (size_t)d * ops->num_faces * nq * ne};
  double *host_out[5] = {out->J_q, out->Lambda_q, out->J_f, out->nJf, out->nJq};
  double *dev_out[5];
  if (memory == SSE_DEVICE) {
    for (int m = 0; m < d; ++m) g.xyz[m] = xyz[m];
    for (int t = 0; t < 5; ++t) dev_out[t] = host_out[t];
  } else {
    for (int m = 0; m < d; ++m)
      if ((e = buf.upload(xyz[m], (size_t)nm * ne, &g.xyz[m])) != cudaSuccess) return cuda(e, "upload xyz");
    for (int t = 0; t < 5; ++t) {
      void *p = nullptr;
      if ((e = buf.alloc(len[t] * sizeof(double), &p)) != cudaSuccess) return cuda(e, "allocate outputs");
      dev_out[t] = (double *)p;
    }
  }
  g.J_q = dev_out[0];
  g.Lambda_q = dev_out[1];
  g.J_f = dev_out[2];
  g.nJf = dev_out[3];
  g.nJq = dev_out[4];

  const int threads = d == 2 ? 32 : 128;
  const dim3 grid((unsigned)n_e);
  if (ops->metrics == SSE_EXACT_METRICS) {
    if (d == 2) {
      cudaFuncSetAttribute(exact_metrics_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      exact_metrics_kernel<2><<<grid, threads, smem>>>(g);
    } else {
      cudaFuncSetAttribute(exact_metrics_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
      exact_metrics_kernel<3><<<grid, threads, smem>>>(g);
    }
  } else if (d == 2) {
    cudaFuncSetAttribute(curl_metrics_2d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    curl_metrics_2d_kernel<<<grid, threads, smem>>>(g);
  } else {
    cudaFuncSetAttribute(curl_metrics_3d_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    curl_metrics_3d_kernel<<<grid, threads, smem>>>(g);
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda(e, "metric kernel launch");
  if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda(e, "metric kernel");
  if (memory == SSE_HOST) {
    for (int t = 0; t < 5; ++t)
      if ((e = cudaMemcpy(host_out[t], dev_out[t], len[t] * sizeof(double), cudaMemcpyDeviceToHost)) != cudaSuccess)
        return cuda(e, "copy geometric factors to the host");
  }
  return SSE_OK;
}

}  // namespace sse
