// sse_abi.cu -- C-ABI of the GB300 residual library (include/sse_gb300.h).
//
// Host side of the drop-in for `Solver{..., GB300}` + `semi_discrete_residual!`
// (src/Solvers/Solvers.jl:259-333, 474-514): validates the caller's operator
// and geometry arrays, converts the Julia CSC matrices into the pair and
// CSR tables the kernels use, keeps everything resident on the device and
// launches the two residual phases on the handle's stream.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <exception>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>  // header-only NVTX ranges (no link dependency)

#include <cuda_runtime.h>

#include "../../include/sse_gb300.h"
#include "sse_kernels.cuh"

using namespace sse;

namespace {

thread_local std::string g_create_error;

// Carpenter & Kennedy (1994), NASA TM-109112: five-stage fourth-order
// 2N-storage Runge-Kutta coefficients (CarpenterKennedy2N54).
const double kCKA[5] = {0.0, -567301805773.0 / 1357537059087.0,
                        -2404267990393.0 / 2016746695238.0,
                        -3550918686646.0 / 2091501179385.0,
                        -1275806237668.0 / 842570457699.0};
const double kCKB[5] = {1432997174477.0 / 9575080441755.0, 5161836677717.0 / 13612068292357.0,
                        1720146321549.0 / 2090206949498.0, 3134564353537.0 / 4481467310338.0,
                        2277821191437.0 / 14882151754819.0};

struct Status {
  int code = SSE_OK;
  std::string msg;
};

struct CsrHost {
  std::vector<int> ptr, idx;
  std::vector<double> val;
};

}  // namespace

struct sse_solver {
  sse_config cfg{};
  KernelArgs ka{};
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  std::vector<void *> allocations;  // device buffers owned by the handle
  double *d_u = nullptr, *d_dudt = nullptr, *d_tmp = nullptr, *d_acc = nullptr, *d_ust = nullptr;
  double *d_partial = nullptr, *d_uf_ref = nullptr;
  int *d_flag = nullptr;
  int *h_flag = nullptr;    // pinned host copy of the flag (read after each call)
  int precision = SSE_FP64;
  std::string last_error;
  // element counts of the device operator arrays (for the FP32 roundings)
  size_t nA = 0, nB = 0, nC = 0, nnzR = 0, nvpS = 0, nfpC = 0, nVd = 0;
  double volume = 0.0;      // sum of W .* J_q over the mesh
  bool mixed_ready = false; // FP32 copies allocated
  bool ref_ready = false;   // reference state of the mixed form chosen
  double *d_comp = nullptr; // compensation of the mixed form's stage accumulation
  double *d_rref = nullptr; // FP64 residual of the mixed form's reference state
  bool compact_ok = false;  // std_compact_kernel applies to this configuration
  double *d_ust2 = nullptr; // second stage buffer of the one-kernel stages
  std::vector<double> h_partial;  // host copy of the per-element sums (sized once)
  // one Runge-Kutta step captured as a CUDA graph, replayed by sse_rk_steps;
  // rebuilt when any of the values it was captured with changes
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    double *u = nullptr;
    double dt = 0.0;
    int scheme = -1, mixed = -1, compact = -1;
    cudaStream_t stream = nullptr;
  } step_graph;
  // discrete adjoint: VJP scratch (allocated on first use)
  bool adj_ready = false;
  bool adj_mixed_ready = false;
  bool mapP_involution = false;  // mapP(mapP(x)) == x: each interface seen from both sides
  int mode0 = -1;                // modal index of the constant basis function (modal V)
  double phi0 = 0.0;             // its (constant) value at the quadrature nodes
  double *d_lam = nullptr, *d_mu = nullptr;
  // trajectory recorded by sse_rk_record for sse_rk_adjoint
  struct Tape {
    bool valid = false;
    int n_steps = 0, every = 0, scheme = 0, stages = 0, nseg = 0;
    int slots_seg = -1;  // segment whose stage data the slots hold
    bool mixed = false;  // recorded (and recomputed) in SSE_MIXED
    bool nodal = false;  // FP64 phase-A outputs kept per stage (FP64 recordings)
    double dt = 0.0;
    size_t bytes = 0;
    void *block = nullptr;     // one device allocation holding every buffer below;
    size_t capacity = 0;       // kept across recordings that fit, freed by sse_destroy
    double *ckpt = nullptr, *ckpt_comp = nullptr;  // nseg states (+ compensation)
    double *seg_y = nullptr, *seg_uq = nullptr, *seg_uf = nullptr;  // every*stages slots
    double *w_u = nullptr, *w_tmp = nullptr, *w_comp = nullptr, *w_dudt = nullptr;
    double *w_acc = nullptr, *w_ust = nullptr;
    double *ybar = nullptr, *qbar = nullptr, *yp = nullptr;
    // binomial schedule (sse_rk_record_binomial): checkpoint slots 0..ckpts
    // (slot 0 the initial state), stage data of one step, the action list of
    // the whole reversal, and how far the recording run carried it
    bool binomial = false;
    int ckpts = 0;
    std::vector<int> plan;   // action kind << 28 | argument
    size_t plan_pos = 0;     // the recorded leaf's action while the descent is intact
    bool descent_intact = false;
    long long plan_steps = 0;  // forward steps the whole action list evaluates
  } tape;
};

namespace {

int fail(sse_solver *s, int code, const std::string &msg) {
  if (s) s->last_error = msg;
  else g_create_error = msg;
  return code;
}

int cuda_fail(sse_solver *s, cudaError_t e, const char *where) {
  return fail(s, SSE_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}

// (uploaded arrays carry the same 64 bytes of slack as alloc's buffers)
template <typename T>
cudaError_t upload(sse_solver *s, const T *host, size_t n, const T **dev) {
  *dev = nullptr;
  if (n == 0) return cudaSuccess;
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, n * sizeof(T) + 64);
  if (e != cudaSuccess) return e;
  s->allocations.push_back(p);
  e = cudaMemcpy(p, host, n * sizeof(T), cudaMemcpyHostToDevice);
  *dev = (const T *)p;
  return e;
}

// Device buffers owned by the handle carry 64 bytes of slack at the end: the
// kernels stage per-element slabs with bulk copies of their 16-byte-aligned
// spans, which may reach up to 15 bytes past the last slab.
cudaError_t alloc(sse_solver *s, size_t bytes, void **out) {
  void *p = nullptr;
  cudaError_t e = cudaMalloc(&p, bytes + 64);
  if (e != cudaSuccess) return e;
  s->allocations.push_back(p);
  *out = p;
  return cudaSuccess;
}

// validate a Julia CSC matrix of the expected shape
bool csc_ok(const sse_csc &A, int64_t m, int64_t n, std::string &why, const char *name) {
  if (A.m != m || A.n != n || !A.colptr) {
    why = std::string(name) + ": expected " + std::to_string(m) + "x" + std::to_string(n) +
          " CSC matrix";
    return false;
  }
  if (A.colptr[0] != 1) { why = std::string(name) + ": colptr must start at 1"; return false; }
  for (int64_t j = 0; j < n; ++j)
    if (A.colptr[j + 1] < A.colptr[j]) { why = std::string(name) + ": colptr not monotone"; return false; }
  int64_t nnz = A.colptr[n] - 1;
  if (nnz > 0 && (!A.rowval || !A.nzval)) { why = std::string(name) + ": null rowval/nzval"; return false; }
  for (int64_t q = 0; q < nnz; ++q)
    if (A.rowval[q] < 1 || A.rowval[q] > m) { why = std::string(name) + ": row index out of range"; return false; }
  return true;
}

// CSC (m x n) -> CSR rows of A (transpose = false) or of A^T (transpose = true)
CsrHost csc_to_csr(const sse_csc &A, bool transpose) {
  CsrHost out;
  int64_t rows = transpose ? A.n : A.m;
  out.ptr.assign(rows + 1, 0);
  int64_t nnz = A.colptr[A.n] - 1;
  if (transpose) {
    for (int64_t j = 0; j < A.n; ++j) {
      for (int64_t q = A.colptr[j] - 1; q < A.colptr[j + 1] - 1; ++q) {
        out.idx.push_back((int)(A.rowval[q] - 1));
        out.val.push_back(A.nzval[q]);
      }
      out.ptr[j + 1] = (int)out.idx.size();
    }
    return out;
  }
  std::vector<int> count(A.m, 0);
  for (int64_t q = 0; q < nnz; ++q) count[A.rowval[q] - 1]++;
  for (int64_t i = 0; i < A.m; ++i) out.ptr[i + 1] = out.ptr[i] + count[i];
  out.idx.resize(nnz);
  out.val.resize(nnz);
  std::vector<int> fill(out.ptr.begin(), out.ptr.end() - 1);
  for (int64_t j = 0; j < A.n; ++j)
    for (int64_t q = A.colptr[j] - 1; q < A.colptr[j + 1] - 1; ++q) {
      int i = (int)(A.rowval[q] - 1);
      out.idx[fill[i]] = (int)j;
      out.val[fill[i]] = A.nzval[q];
      fill[i]++;
    }
  return out;
}

int upload_csr(sse_solver *s, const CsrHost &c, const int **ptr, const int **idx, const double **val) {
  cudaError_t e;
  if ((e = upload(s, c.ptr.data(), c.ptr.size(), ptr)) != cudaSuccess) return cuda_fail(s, e, "upload");
  if ((e = upload(s, c.idx.data(), c.idx.size(), idx)) != cudaSuccess) return cuda_fail(s, e, "upload");
  if ((e = upload(s, c.val.data(), c.val.size(), val)) != cudaSuccess) return cuda_fail(s, e, "upload");
  return SSE_OK;
}

size_t geo_len(const sse_config &c, int what) {
  size_t d = c.d, nq = c.n_q, nf = c.n_f, ne = c.n_e;
  switch (what) {
    case 0: return nf * ne;                 // BJf
    case 1: return d * nf * ne;             // n_f
    case 2: return nq * d * d * ne;         // halfWLambda / Lambda_q
    case 3: return nq * ne;                 // WJ / JinvW / WJinv
    case 4: return d * nf * ne;             // halfnJf
    case 5: return d * c.num_faces * nq * ne;  // halfnJq
  }
  return 0;
}

// dense rows x cols copy of a Julia CSC matrix (column-major)
std::vector<double> csc_dense(const sse_csc &A, int rows, int cols) {
  std::vector<double> out((size_t)rows * cols, 0.0);
  for (int j = 0; j < cols; ++j)
    for (int64_t q = A.colptr[j] - 1; q < A.colptr[j + 1] - 1; ++q)
      out[(size_t)j * rows + (A.rowval[q] - 1)] += A.nzval[q];
  return out;
}

// The one-kernel StandardForm path (std_compact_kernel): StandardForm on
// elements with at most 32 volume, facet and modal nodes, each face meeting
// one neighbour element, with the element's dense weight-adjusted mass
// operator or a diagonal mass matrix.  Packs V, R V, V^T, R, R^T, D_m and
// D_m^T column-major (leading dimension = rows) and turns the path on; a
// configuration outside that scope keeps the two-phase kernels.
int setup_compact(sse_solver *s, const sse_operators *ops, const std::vector<int> &mapP) {
  const sse_config &c = s->cfg;
  KernelArgs &ka = s->ka;
  const int np = c.n_p, nq = c.n_q, nf = c.n_f, d = c.d, nc = c.n_c;
  const int npf = c.nodes_per_face, nfac = c.num_faces;
  ka.compact = 0;
  s->compact_ok = false;
  if (ka.fd || nq > 32 || nf > 32 || np > 32) return SSE_OK;
  if (ka.mass_wa ? !ka.Ak : !ka.geo.WJinv) return SSE_OK;
  for (int64_t k = 0; k < c.n_e; ++k)
    for (int f = 0; f < nfac; ++f) {
      const size_t b = (size_t)k * nf + (size_t)f * npf;
      for (int j = 1; j < npf; ++j)
        if (mapP[b + j] / nf != mapP[b] / nf) return SSE_OK;
    }
  const bool has_vdm = ka.op.has_vdm != 0;
  cudaError_t e;
  std::vector<double> V;
  if (has_vdm) {
    V.resize((size_t)nq * np);
    if (ka.op.dense_v) {
      std::memcpy(V.data(), ops->V_dense, V.size() * sizeof(double));
    } else {
      void *p;
      if ((e = alloc(s, V.size() * sizeof(double), &p))) return cuda_fail(s, e, "alloc dense V");
      if ((e = launch_dense_vdm(ka, (double *)p, s->stream)) ||
          (e = cudaMemcpyAsync(V.data(), p, V.size() * sizeof(double), cudaMemcpyDeviceToHost, s->stream)) ||
          (e = cudaStreamSynchronize(s->stream)))
        return cuda_fail(s, e, "dense V");
    }
  }
  const std::vector<double> R = csc_dense(ops->R, nf, nq);
  std::vector<double> VR((size_t)nf * np, 0.0);  // R V (R when V = I)
  for (int a = 0; a < np; ++a)
    for (int j = 0; j < nf; ++j) {
      double acc = 0.0;
      if (has_vdm)
        for (int q = 0; q < nq; ++q) acc += R[(size_t)q * nf + j] * V[(size_t)a * nq + q];
      else
        acc = R[(size_t)a * nf + j];
      VR[(size_t)a * nf + j] = acc;
    }
  std::vector<double> pack;
  std::vector<int> ipack;
  auto region = [&](int slot, const std::vector<double> &m) {
    ka.cop_off[slot] = (int)pack.size();
    pack.insert(pack.end(), m.begin(), m.end());
    if (pack.size() & 1) pack.push_back(0.0);
  };
  // a sparse operator (rows x cols, column-major dense copy m) as padded
  // rows: its k-th nonzero of row r at [k * rows + r] in increasing column
  // order, the column index beside it; kept dense when the widest row holds
  // more than three quarters of the columns
  auto sparse_region = [&](int slot, const std::vector<double> &m, int rows, int cols) {
    std::vector<std::vector<int>> nz(rows);
    size_t w = 0;
    for (int r = 0; r < rows; ++r) {
      for (int q = 0; q < cols; ++q)
        if (m[(size_t)q * rows + r] != 0.0) nz[r].push_back(q);
      w = std::max(w, nz[r].size());
    }
    if (4 * w > (size_t)3 * cols || w == 0) {
      ka.cop_w[slot] = 0;
      region(slot, m);
      return;
    }
    std::vector<double> val(w * rows, 0.0);
    std::vector<int> idx(w * rows, 0);
    for (int r = 0; r < rows; ++r)
      for (size_t k = 0; k < nz[r].size(); ++k) {
        val[k * rows + r] = m[(size_t)nz[r][k] * rows + r];
        idx[k * rows + r] = nz[r][k];
      }
    ka.cop_w[slot] = (int)w;
    ka.cop_i[slot] = (int)ipack.size();
    ipack.insert(ipack.end(), idx.begin(), idx.end());
    region(slot, val);
  };
  for (int i = 0; i < 12; ++i) { ka.cop_off[i] = 0; ka.cop_w[i] = 0; ka.cop_i[i] = 0; }
  if (has_vdm) {
    region(kCopV, V);
    std::vector<double> VT((size_t)np * nq);
    for (int i = 0; i < nq; ++i)
      for (int a = 0; a < np; ++a) VT[(size_t)i * np + a] = V[(size_t)a * nq + i];
    region(kCopVT, VT);
  }
  region(kCopVR, VR);
  sparse_region(kCopR, R, nf, nq);
  {
    std::vector<double> RT((size_t)nq * nf);
    for (int j = 0; j < nf; ++j)
      for (int i = 0; i < nq; ++i) RT[(size_t)j * nq + i] = R[(size_t)i * nf + j];
    sparse_region(kCopRT, RT, nq, nf);
  }
  for (int m = 0; m < d; ++m) {
    const std::vector<double> Dm = csc_dense(ops->D[m], nq, nq);
    std::vector<double> DT((size_t)nq * nq);
    for (int q = 0; q < nq; ++q)
      for (int i = 0; i < nq; ++i) DT[(size_t)q * nq + i] = Dm[(size_t)i * nq + q];
    sparse_region(kCopD + m, Dm, nq, nq);
    sparse_region(kCopDT + m, DT, nq, nq);
  }
  ka.cop_doubles = (int)pack.size();
  while (ipack.size() & 3) ipack.push_back(0);
  ka.copi_ints = (int)ipack.size();
  const size_t ops_doubles = (size_t)ka.cop_doubles + ka.copi_ints / 2;
  // per-element regions
  const int sizes[10] = {(1 + nfac) * nc * np, 0, nc * nq, d * nc * nq, d * nc * nq, nc * nf, nc * nq, nc * np,
                         d * d * nq + 4,       ka.mass_wa ? np * np + 4 : 0};
  int off = 0;
  for (int i = 0; i < 10; ++i) { ka.ct_off[i] = off; off += (sizes[i] + 1) & ~1; }
  ka.ct_doubles = off;
  // four elements (warps) per block; fewer when shared memory is short
  const size_t cap = 220 * 1024;
  int epb = std::min(4, kMaxCompactEpb);
  while (epb > 1 && (ops_doubles + (size_t)epb * ka.ct_doubles) * 8 > cap) epb /= 2;
  if ((ops_doubles + (size_t)epb * ka.ct_doubles) * 8 > cap) return SSE_OK;
  ka.epb_c = epb;
  if ((e = upload(s, pack.data(), pack.size(), &ka.cops))) return cuda_fail(s, e, "upload compact operators");
  ka.copi = nullptr;
  if (!ipack.empty() && (e = upload(s, ipack.data(), ipack.size(), &ka.copi)))
    return cuda_fail(s, e, "upload compact operators");
  if ((e = sse_set_smem_limit_compact(ka, (ops_doubles + (size_t)epb * ka.ct_doubles) * 8)))
    return cuda_fail(s, e, "cudaFuncSetAttribute");
  s->compact_ok = true;
  ka.compact = 1;
  return SSE_OK;
}

int build(sse_solver *s, const sse_config *cfg, const sse_operators *ops, const sse_geometry *geo) {
  const sse_config &c = *cfg;
  std::string why;
  if (!(c.d == 2 || c.d == 3)) return fail(s, SSE_ERR_UNSUPPORTED, "d must be 2 or 3");
  if (!((c.law == SSE_LINEAR_ADVECTION && c.n_c == 1) || (c.law == SSE_EULER && c.n_c == c.d + 2)))
    return fail(s, SSE_ERR_UNSUPPORTED, "law / n_c combination not supported");
  if (c.n_p <= 0 || c.n_q <= 0 || c.n_f <= 0 || c.n_e <= 0 || c.num_faces <= 0 ||
      c.nodes_per_face * c.num_faces != c.n_f)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "invalid sizes in sse_config");
  if (c.n_q > 65535 || c.n_f > 65535) return fail(s, SSE_ERR_UNSUPPORTED, "n_q, n_f must be < 65536");
  if (c.form != SSE_STANDARD_FORM && c.form != SSE_FLUX_DIFFERENCING_FORM)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "unknown form");
  if (c.numerical_flux < 0 || c.numerical_flux > 2) return fail(s, SSE_ERR_INVALID_ARGUMENT, "unknown numerical flux");
  if (c.two_point_flux < 0 || c.two_point_flux > 2) return fail(s, SSE_ERR_INVALID_ARGUMENT, "unknown two-point flux");
  if (c.mass_solver != SSE_WEIGHT_ADJUSTED && c.mass_solver != SSE_DIAGONAL)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "unknown mass solver");
  if (c.law == SSE_EULER && !(c.gamma > 1.0)) return fail(s, SSE_ERR_INVALID_ARGUMENT, "gamma must exceed 1");
  if ((double)c.n_f * c.n_e > 2.0e9 || (double)c.n_q * c.n_c * c.n_e > 4.0e18)
    return fail(s, SSE_ERR_UNSUPPORTED, "mesh too large for 32-bit facet indices");
  const bool fd = c.form == SSE_FLUX_DIFFERENCING_FORM;
  const bool dense_v = ops->V_dense != nullptr;
  if (dense_v && (ops->vdm_A || ops->vdm_B || ops->vdm_C))
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "give V either as warped tensor-product factors or dense, not both");
  const bool has_vdm = ops->vdm_A != nullptr || dense_v;
  if (!has_vdm && c.n_p != c.n_q) return fail(s, SSE_ERR_INVALID_ARGUMENT, "V = I requires n_p == n_q");
  if (c.mass_solver == SSE_WEIGHT_ADJUSTED && !has_vdm)
    return fail(s, SSE_ERR_UNSUPPORTED, "WeightAdjustedSolver requires a modal V");
  if (!geo->BJf || !geo->n_f || !geo->mapP || !geo->WJ)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "geometry: BJf, n_f, mapP and WJ are required");
  if (c.mass_solver == SSE_WEIGHT_ADJUSTED && !geo->JinvW)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "geometry: JinvW required for WeightAdjustedSolver");
  if (c.mass_solver == SSE_DIAGONAL && !geo->WJinv)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "geometry: WJinv required for DiagonalSolver");
  if (fd && c.law == SSE_EULER && has_vdm && !geo->JinvW)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "geometry: JinvW required for the entropy projection");
  if (fd && (!geo->Lambda_q || !geo->halfnJf || !geo->halfnJq))
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "geometry: Lambda_q, halfnJf, halfnJq required for FluxDifferencingForm");
  if (!fd && !geo->halfWLambda)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "geometry: halfWLambda required for StandardForm");
  if (!csc_ok(ops->R, c.n_f, c.n_q, why, "R")) return fail(s, SSE_ERR_INVALID_ARGUMENT, why);
  for (int m = 0; m < c.d; ++m) {
    if (fd) {
      if (!csc_ok(ops->S[m], c.n_q, c.n_q, why, "S")) return fail(s, SSE_ERR_INVALID_ARGUMENT, why);
    } else if (!csc_ok(ops->D[m], c.n_q, c.n_q, why, "D")) {
      return fail(s, SSE_ERR_INVALID_ARGUMENT, why);
    }
  }
  const bool has_C = fd && ops->C.colptr && ops->C.n > 0;
  if (has_C && !csc_ok(ops->C, c.n_q, c.n_f, why, "C")) return fail(s, SSE_ERR_INVALID_ARGUMENT, why);

  // ---- warped tensor-product factors (validated before any device work)
  int p1 = 0, M1 = 0, M2 = 0, M3 = 1;
  std::vector<int> sigma, modes, b12, b12_index;
  if (dense_v) {
    // the constant mode of a multidimensional orthonormal basis: the column
    // of V that is the same at every volume node
    M3 = 0;
    for (int a = 0; a < c.n_p && s->mode0 < 0; ++a) {
      const double *col = ops->V_dense + (size_t)c.n_q * a;
      bool same = std::isfinite(col[0]) && std::fabs(col[0]) > 0.0;
      for (int i = 1; i < c.n_q && same; ++i)
        same = std::fabs(col[i] - col[0]) <= 1e-12 * std::fabs(col[0]);
      if (same) { s->mode0 = a; s->phi0 = col[0]; }
    }
    for (size_t t = 0; t < (size_t)c.n_q * c.n_p; ++t)
      if (!std::isfinite(ops->V_dense[t])) return fail(s, SSE_ERR_INVALID_ARGUMENT, "V_dense is not finite");
  } else if (has_vdm) {
    p1 = ops->vdm_p + 1;
    M1 = ops->vdm_m[0]; M2 = ops->vdm_m[1]; M3 = c.d == 3 ? ops->vdm_m[2] : 1;
    if (p1 < 1 || p1 > 16 || M1 < 1 || M2 < 1 || M3 < 1 || M1 * M2 * M3 != c.n_q || !ops->vdm_B ||
        !ops->vdm_sigma_in || (c.d == 3 && !ops->vdm_C))
      return fail(s, SSE_ERR_INVALID_ARGUMENT, "inconsistent warped tensor-product factors");
    size_t nsig = (size_t)p1 * p1 * (c.d == 3 ? p1 : 1);
    sigma.assign(nsig, -1);
    modes.assign(c.n_p, -1);
    b12_index.assign((size_t)p1 * p1, -1);
    int count = 0;
    for (size_t t = 0; t < nsig; ++t) {
      int64_t l = ops->vdm_sigma_in[t];
      if (l < 0 || l > c.n_p) return fail(s, SSE_ERR_INVALID_ARGUMENT, "sigma_in out of range");
      if (l == 0) continue;
      int b1 = (int)(t % p1), b2 = (int)((t / p1) % p1), b3 = c.d == 3 ? (int)(t / (p1 * p1)) : 0;
      if (b1 + b2 + b3 >= p1) return fail(s, SSE_ERR_INVALID_ARGUMENT, "sigma_in outside the simplex");
      if (modes[l - 1] != -1) return fail(s, SSE_ERR_INVALID_ARGUMENT, "sigma_in repeats a mode");
      sigma[t] = (int)(l - 1);
      modes[l - 1] = b1 | (b2 << 8) | (b3 << 16);
      ++count;
    }
    if (count != c.n_p) return fail(s, SSE_ERR_INVALID_ARGUMENT, "sigma_in must enumerate n_p modes");
    for (int b1 = 0; b1 < p1; ++b1)
      for (int b2 = 0; b1 + b2 < p1; ++b2) {
        b12_index[b1 + p1 * b2] = (int)b12.size();
        b12.push_back(b1 | (b2 << 8));
      }
    // the constant mode (b1, b2, b3) = 0: its value is the product of the
    // first entries of the 1-D factors (each constant in its node index)
    s->mode0 = sigma[0];
    s->phi0 = ops->vdm_A[0] * ops->vdm_B[0] * (c.d == 3 ? ops->vdm_C[0] : 1.0);
    if (s->mode0 < 0 || !(std::fabs(s->phi0) > 0.0))
      return fail(s, SSE_ERR_INVALID_ARGUMENT, "the modal basis has no constant mode");
  }
  // ---- connectivity (validated before any device work)
  std::vector<int> mapP((size_t)c.n_f * c.n_e);
  {
    const int64_t lim = (int64_t)c.n_f * c.n_e;
    for (size_t t = 0; t < mapP.size(); ++t) {
      int64_t P = geo->mapP[t];
      if (P < 1 || P > lim) return fail(s, SSE_ERR_INVALID_ARGUMENT, "mapP index out of range");
      mapP[t] = (int)(P - 1);
    }
    s->mapP_involution = true;
    for (size_t t = 0; t < mapP.size(); ++t)
      if ((size_t)mapP[mapP[t]] != t) { s->mapP_involution = false; break; }
  }

  s->cfg = c;
  KernelArgs &ka = s->ka;
  DevOps &op = ka.op;
  op.d = c.d; op.nc = c.n_c; op.np = c.n_p; op.nq = c.n_q; op.nf = c.n_f;
  op.nfac = c.num_faces; op.npf = c.nodes_per_face;
  cudaError_t e;

  op.has_vdm = has_vdm;
  op.dense_v = dense_v;
  if (dense_v) {
    op.p1 = 0; op.M1 = 0; op.M2 = 0; op.M3 = 0; op.nb12 = 0;
    if ((e = upload(s, ops->V_dense, (size_t)c.n_q * c.n_p, &op.Vd)) != cudaSuccess)
      return cuda_fail(s, e, "upload V_dense");
    s->nVd = (size_t)c.n_q * c.n_p;
  } else if (has_vdm) {
    op.p1 = p1; op.M1 = M1; op.M2 = M2; op.M3 = M3;
    op.nb12 = (int)b12.size();
    if ((e = upload(s, ops->vdm_A, (size_t)M1 * p1, &op.A)) != cudaSuccess) return cuda_fail(s, e, "upload A");
    if ((e = upload(s, ops->vdm_B, (size_t)M2 * p1 * p1, &op.B)) != cudaSuccess) return cuda_fail(s, e, "upload B");
    if (c.d == 3 && (e = upload(s, ops->vdm_C, (size_t)M3 * p1 * p1 * p1, &op.C)) != cudaSuccess)
      return cuda_fail(s, e, "upload C");
    if ((e = upload(s, sigma.data(), sigma.size(), &op.sigma)) != cudaSuccess) return cuda_fail(s, e, "upload");
    if ((e = upload(s, modes.data(), modes.size(), &op.modes)) != cudaSuccess) return cuda_fail(s, e, "upload");
    if ((e = upload(s, b12.data(), b12.size(), &op.b12)) != cudaSuccess) return cuda_fail(s, e, "upload");
    if ((e = upload(s, b12_index.data(), b12_index.size(), &op.b12_index)) != cudaSuccess)
      return cuda_fail(s, e, "upload");
    s->nA = (size_t)M1 * p1;
    s->nB = (size_t)M2 * p1 * p1;
    s->nC = c.d == 3 ? (size_t)M3 * p1 * p1 * p1 : 0;
  }
  s->nnzR = (size_t)(ops->R.colptr[ops->R.n] - 1);
  for (size_t t = 0; t < (size_t)c.n_q * c.n_e; ++t) s->volume += geo->WJ[t];

  // ---- the tables of the FP64 logarithm and exponential of the entropy maps
  {
    std::vector<double> mt(3 * kLogTab + 2 * kExpTab);
    sse_build_math_tables(mt.data());
    if ((e = upload(s, mt.data(), mt.size(), &op.math_tab)) != cudaSuccess) return cuda_fail(s, e, "upload");
  }

  // ---- R, R^T, D, D^T
  int rc;
  if ((rc = upload_csr(s, csc_to_csr(ops->R, false), &op.R_ptr, &op.R_idx, &op.R_val))) return rc;
  if ((rc = upload_csr(s, csc_to_csr(ops->R, true), &op.Rt_ptr, &op.Rt_idx, &op.Rt_val))) return rc;
  if (!fd) {
    for (int m = 0; m < c.d; ++m) {
      if ((rc = upload_csr(s, csc_to_csr(ops->D[m], false), &op.D_ptr[m], &op.D_idx[m], &op.D_val[m]))) return rc;
      if ((rc = upload_csr(s, csc_to_csr(ops->D[m], true), &op.Dt_ptr[m], &op.Dt_idx[m], &op.Dt_val[m]))) return rc;
    }
  }

  // ---- flux-differencing pair tables
  if (fd) {
    // unique pairs (i < j) over the union of the S_m patterns, ordered by (j, i)
    std::vector<std::pair<int, int>> pairs;
    for (int m = 0; m < c.d; ++m) {
      const sse_csc &S = ops->S[m];
      for (int64_t j = 0; j < S.n; ++j)
        for (int64_t q = S.colptr[j] - 1; q < S.colptr[j + 1] - 1; ++q) {
          int i = (int)(S.rowval[q] - 1);
          if (i < j) pairs.emplace_back((int)j, i);
        }
    }
    std::sort(pairs.begin(), pairs.end());
    pairs.erase(std::unique(pairs.begin(), pairs.end()), pairs.end());
    const int nvp = (int)pairs.size();
    std::vector<int> vp_ij(nvp);
    std::vector<double> vp_S((size_t)nvp * c.d, 0.0);
    for (int t = 0; t < nvp; ++t) vp_ij[t] = pairs[t].second | (pairs[t].first << 16);
    for (int m = 0; m < c.d; ++m) {
      const sse_csc &S = ops->S[m];
      for (int64_t j = 0; j < S.n; ++j)
        for (int64_t q = S.colptr[j] - 1; q < S.colptr[j + 1] - 1; ++q) {
          int i = (int)(S.rowval[q] - 1);
          if (i >= j) continue;
          auto it = std::lower_bound(pairs.begin(), pairs.end(), std::make_pair((int)j, i));
          vp_S[(size_t)(it - pairs.begin()) * c.d + m] = S.nzval[q];
        }
    }
    std::vector<std::vector<int>> inc(c.n_q);
    for (int t = 0; t < nvp; ++t) {
      inc[pairs[t].second].push_back((t << 1) | 1);
      inc[pairs[t].first].push_back(t << 1);
    }
    std::vector<int> inc_ptr(c.n_q + 1, 0), inc_flat;
    for (int i = 0; i < c.n_q; ++i) {
      inc_flat.insert(inc_flat.end(), inc[i].begin(), inc[i].end());
      inc_ptr[i + 1] = (int)inc_flat.size();
    }
    op.nvp = nvp;
    s->nvpS = (size_t)nvp * c.d;
    if ((e = upload(s, vp_ij.data(), vp_ij.size(), &op.vp_ij)) != cudaSuccess) return cuda_fail(s, e, "upload");
    if ((e = upload(s, vp_S.data(), vp_S.size(), &op.vp_S)) != cudaSuccess) return cuda_fail(s, e, "upload");
    {
      // S / 2 (exact): the forward EC pair flux takes its metric vector halved
      std::vector<double> half(vp_S);
      for (double &v : half) v *= 0.5;
      if ((e = upload(s, half.data(), half.size(), &op.vp_Sh)) != cudaSuccess) return cuda_fail(s, e, "upload");
    }
    if ((e = upload(s, inc_ptr.data(), inc_ptr.size(), &op.vp_inc_ptr)) != cudaSuccess) return cuda_fail(s, e, "upload");
    if ((e = upload(s, inc_flat.data(), inc_flat.size(), &op.vp_inc)) != cudaSuccess) return cuda_fail(s, e, "upload");

    op.nfp = 0;
    if (has_C) {
      const sse_csc &Cm = ops->C;
      std::vector<int> fp_ij;
      std::vector<double> fp_C;
      std::vector<std::vector<int>> qinc(c.n_q), finc(c.n_f);
      for (int64_t j = 0; j < Cm.n; ++j)
        for (int64_t q = Cm.colptr[j] - 1; q < Cm.colptr[j + 1] - 1; ++q) {
          int i = (int)(Cm.rowval[q] - 1);
          int t = (int)fp_ij.size();
          fp_ij.push_back(i | ((int)j << 16));
          fp_C.push_back(Cm.nzval[q]);
          qinc[i].push_back(t);
          finc[j].push_back(t);
        }
      std::vector<int> qptr(c.n_q + 1, 0), qflat, fptr(c.n_f + 1, 0), fflat;
      for (int i = 0; i < c.n_q; ++i) { qflat.insert(qflat.end(), qinc[i].begin(), qinc[i].end()); qptr[i + 1] = (int)qflat.size(); }
      for (int j = 0; j < c.n_f; ++j) { fflat.insert(fflat.end(), finc[j].begin(), finc[j].end()); fptr[j + 1] = (int)fflat.size(); }
      op.nfp = (int)fp_ij.size();
      s->nfpC = fp_C.size();
      if ((e = upload(s, fp_ij.data(), fp_ij.size(), &op.fp_ij)) != cudaSuccess) return cuda_fail(s, e, "upload");
      if ((e = upload(s, fp_C.data(), fp_C.size(), &op.fp_C)) != cudaSuccess) return cuda_fail(s, e, "upload");
      {
        std::vector<double> half(fp_C);
        for (double &v : half) v *= 0.5;
        if ((e = upload(s, half.data(), half.size(), &op.fp_Ch)) != cudaSuccess) return cuda_fail(s, e, "upload");
      }
      if ((e = upload(s, qptr.data(), qptr.size(), &op.fp_q_ptr)) != cudaSuccess) return cuda_fail(s, e, "upload");
      if ((e = upload(s, qflat.data(), qflat.size(), &op.fp_q)) != cudaSuccess) return cuda_fail(s, e, "upload");
      if ((e = upload(s, fptr.data(), fptr.size(), &op.fp_f_ptr)) != cudaSuccess) return cuda_fail(s, e, "upload");
      if ((e = upload(s, fflat.data(), fflat.size(), &op.fp_f)) != cudaSuccess) return cuda_fail(s, e, "upload");
    }
  }

  // ---- geometry
  DevGeo &g = ka.geo;
  if ((e = upload(s, mapP.data(), mapP.size(), &g.mapP)) != cudaSuccess) return cuda_fail(s, e, "upload mapP");
  if ((e = upload(s, geo->BJf, geo_len(c, 0), &g.BJf)) != cudaSuccess) return cuda_fail(s, e, "upload BJf");
  if ((e = upload(s, geo->n_f, geo_len(c, 1), &g.n_f)) != cudaSuccess) return cuda_fail(s, e, "upload n_f");
  if ((e = upload(s, geo->WJ, geo_len(c, 3), &g.WJ)) != cudaSuccess) return cuda_fail(s, e, "upload WJ");
  if (geo->JinvW && (e = upload(s, geo->JinvW, geo_len(c, 3), &g.JinvW)) != cudaSuccess) return cuda_fail(s, e, "upload");
  if (geo->WJinv && (e = upload(s, geo->WJinv, geo_len(c, 3), &g.WJinv)) != cudaSuccess) return cuda_fail(s, e, "upload");
  if (fd) {
    if ((e = upload(s, geo->Lambda_q, geo_len(c, 2), &g.Lambda_q)) != cudaSuccess) return cuda_fail(s, e, "upload");
    if ((e = upload(s, geo->halfnJf, geo_len(c, 4), &g.halfnJf)) != cudaSuccess) return cuda_fail(s, e, "upload");
    if ((e = upload(s, geo->halfnJq, geo_len(c, 5), &g.halfnJq)) != cudaSuccess) return cuda_fail(s, e, "upload");
  } else {
    if ((e = upload(s, geo->halfWLambda, geo_len(c, 2), &g.halfWLambda)) != cudaSuccess) return cuda_fail(s, e, "upload");
  }

  // ---- physics
  Physics &ph = ka.ph;
  ph.law = c.law;
  ph.nflux = c.numerical_flux;
  ph.ec = (c.two_point_flux == SSE_EC_FLUX) ? 1 : 0;
  ph.chandrashekar = (c.two_point_flux == SSE_CHANDRASHEKAR_FLUX) ? 1 : 0;
  ph.half_lambda = c.half_lambda;
  ph.gamma = c.gamma;
  ph.gm1 = c.gamma - 1.0;
  ph.igm1 = c.law == SSE_EULER ? 1.0 / (c.gamma - 1.0) : 0.0;
  ph.ilm_q[0] = ph.igm1 * 2.0;
  ph.ilm_q[1] = ph.igm1 * (2.0 / 3.0);
  ph.ilm_q[2] = ph.igm1 * 0.4;
  ph.ilm_q[3] = ph.igm1 * (2.0 / 7.0);
  ph.log_gm1 = c.law == SSE_EULER ? std::log(c.gamma - 1.0) : 0.0;
  for (int m = 0; m < 3; ++m) ph.a[m] = c.a[m];
  ka.fd = fd;
  ka.project_entropy = fd && c.law == SSE_EULER;
  ka.mass_wa = c.mass_solver == SSE_WEIGHT_ADJUSTED;
  ka.ne = c.n_e;

  // ---- team geometry and shared-memory layouts
  const int nc = c.n_c, np = c.n_p, nq = c.n_q, nf = c.n_f, d = c.d;
  // Tets: one element per block, 256 threads once the element has more than
  // 192 volume and facet nodes (measured against 128 threads: phase B 7.6 %
  // and 5.4 % faster at p = 4 and 5, mixed phase A 1.75x -- the FP64 pipe
  // idles less with eight warps per element -- but 15 % slower at p = 3,
  // whose 128 nodes leave half the threads idle).  Small elements: 128-thread
  // blocks of 32-thread teams (measured against 64 x 4 and 32 x 8), or of
  // 16-thread teams for flux differencing on triangles whose volume and
  // facet nodes fit in the node slots of 16 threads: two teams share a warp,
  // so loops over N_p or N_f outputs leave fewer lanes of each warp idle
  // (2-D vortex at p = 4: phase A 0.212 -> 0.178 ms, phase B 0.428 -> 0.396
  // ms; at p = 2 on tets phase B was 43 % slower, and the StandardForm
  // advection mesh of 512 triangles would fill half as many SMs).
  const bool narrow = d == 2 && fd && nq + nf <= kMaxNodeSlots * 16;
  const int tpe = nq < 64 ? (narrow ? 16 : 32) : (nq + nf > 192 ? 256 : 128);
  auto epb_for = [](int tpe_) { return tpe_ < 128 ? 128 / tpe_ : 1; };
  // doubles of shared memory per element team that keep two blocks per SM
  auto team_budget = [&](int tpe_) { return (int)((size_t)110 * 1024 / 8 / epb_for(tpe_)); };
  if (nq + nf > kMaxNodeSlots * tpe)
    return fail(s, SSE_ERR_UNSUPPORTED, "n_q + n_f too large for one element team");
  int zsz = 0, wsz = 0;
  if (has_vdm) {
    if (d == 2) zsz = nc * op.p1 * op.M2;
    else { zsz = nc * op.nb12 * op.M3; wsz = nc * op.p1 * op.M2 * op.M3; }
  }
  auto finish = [](Layout &L, std::initializer_list<int> sizes) {
    int off = 0, i = 0;
    for (int sz : sizes) { L.off[i++] = off; off += (sz + 1) & ~1; }
    for (; i < 12; ++i) L.off[i] = off;
    L.team_doubles = off;
  };
  // phase-A layout: X, Y, Z, W, F, lane partials; F holds NC x max(N_p, N_q,
  // N_f) (modal scratch, facet values, or V dudt in the conservation kernel)
  finish(ka.layA, {nc * std::max(np, nq), nc * nq, zsz, wsz, nc * std::max({np, nq, nf}), tpe * (nc + 1)});
  // energy_kernel: X, Y, Z, W as in phase A, the element mass operator, dudt
  finish(ka.layE, {nc * std::max(np, nq), nc * nq, zsz, wsz, np * np, nc * np});
  if (fd) {
    // the pair buffer holds one chunk of per-pair contributions, and after
    // the pair passes the modal / nodal buffers and the sum-factorisation
    // scratch of the lift: chunks as large as that region (at least 256
    // pairs when there are that many)
    const int zsz_e = (zsz + 1) & ~1;
    const int final_scratch = nc * (np + nq) + zsz_e + wsz;
    const int max_pairs = std::max(op.nvp, op.nfp);
    const int prim = (c.law == SSE_EULER) ? (nq + nf) * (3 + d) : 0;
    auto layout = [&](int chunk) {
      finish(ka.layB, {nc * nq, nc * nf, nc * nf, nc * nq, std::max(chunk * nc, final_scratch),
                       d * d * nq, op.nfp > 0 ? d * c.num_faces * nq : 0, prim});
      return ka.layB.team_doubles;
    };
    // all pairs at once when two blocks still fit on an SM (measured faster
    // than more, smaller blocks with chunked passes); otherwise the largest
    // chunk, a whole number of passes of the element's threads, that does
    const int budget = team_budget(tpe);
    int chunk = max_pairs;
    if (layout(chunk) > budget) {
      // chunks of at least one pass of the element's threads: two blocks per
      // SM when that leaves room for them, else one block per SM
      const int fixed = layout(0) - ((std::max(0, final_scratch) + 1) & ~1);
      const int cap1 = (int)((size_t)220 * 1024 / 8 / epb_for(tpe));
      int room = budget - fixed;
      if (room / nc < std::min(tpe, max_pairs)) room = cap1 - fixed;
      chunk = std::max(1, room / nc);
      if (chunk >= tpe) chunk = chunk / tpe * tpe;
      chunk = std::max(1, std::min(chunk, max_pairs));
    }
    ka.fd_chunk = chunk;
    ka.vdm_zsz = zsz_e;
    layout(chunk);
    // the interface flux of one facet node costs about 0.8 of a volume pair
    // (block timings at p = 4): balance lanes when all pairs are one chunk.
    // Teams narrower than a warp share warps, and a warp waits for its
    // slowest lane: there the split is kept only when the lanes left for the
    // rest of the pairs finish no later than all lanes taking the pairs and
    // the interface flux in turn
    ka.vp_split = 0;
    if (chunk >= op.nvp && nf < tpe && op.nvp > 0) {
      const double unit = (op.nvp + 0.8 * nf) / tpe;
      int a = (int)std::lround(unit - 0.8);
      a = std::max(0, std::min(a, op.nvp / nf));
      if (tpe < 32) {
        const int rest = tpe - nf;
        const double split_cost = std::max(a + 0.8, (double)((op.nvp - a * nf + rest - 1) / rest));
        const double plain_cost = (double)((op.nvp + tpe - 1) / tpe) + 0.8;
        if (split_cost > plain_cost) a = 0;
      }
      ka.vp_split = a;
    }
  } else {
    finish(ka.layB, {nc * nq, nc * nf, nc * nf, nc * nq, d * nc * nq, nc * nq, nc * nq, 0, zsz, wsz});
  }
  int epb = epb_for(tpe);
  const size_t smem_cap = 220 * 1024;
  while (epb > 1 && (size_t)epb * std::max(ka.layA.team_doubles, ka.layB.team_doubles) * 8 > smem_cap) epb /= 2;
  if ((size_t)epb * std::max(ka.layA.team_doubles, ka.layB.team_doubles) * 8 > smem_cap)
    return fail(s, SSE_ERR_UNSUPPORTED, "element too large for shared memory");
  ka.epb = epb;
  ka.tpb = epb * tpe;

  // ---- scratch and state buffers
  size_t nstate = (size_t)np * nc * c.n_e;
  void *p;
  if ((e = alloc(s, (size_t)nq * nc * c.n_e * 8, &p))) return cuda_fail(s, e, "alloc u_q");
  ka.u_q = (double *)p;
  if ((e = alloc(s, (size_t)nf * nc * c.n_e * 8, &p))) return cuda_fail(s, e, "alloc u_f");
  ka.u_f = (double *)p;
  if ((e = alloc(s, nstate * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_u = (double *)p;
  if ((e = alloc(s, nstate * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_dudt = (double *)p;
  if ((e = alloc(s, nstate * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_tmp = (double *)p;
  if ((e = alloc(s, (size_t)c.n_e * (nc + 1) * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_partial = (double *)p;
  if ((e = alloc(s, sizeof(int), &p))) return cuda_fail(s, e, "alloc"); s->d_flag = (int *)p;
  ka.flag = s->d_flag;
  if ((e = cudaMemset(s->d_flag, 0, sizeof(int)))) return cuda_fail(s, e, "memset");
  if ((e = cudaHostAlloc((void **)&s->h_flag, sizeof(int), cudaHostAllocDefault))) return cuda_fail(s, e, "pinned flag");
  *s->h_flag = 0;
  if ((e = cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking))) return cuda_fail(s, e, "stream");
  s->own_stream = true;

  // phase A on 128-thread teams, two elements per block, where phase B uses
  // 256 threads and the element's volume and facet nodes fit in two passes
  // of 128 (p = 4 tets: 3.14 -> 3.09 ms per stage, fewer barrier stalls)
  ka.epb_a = (tpe >= 256 && nq + nf <= 256) ? epb * (tpe / 128) : epb;
  if ((size_t)ka.epb_a * ka.layA.team_doubles * 8 > 220 * 1024) ka.epb_a = epb;
  // opt in to large dynamic shared memory for every kernel instantiation used
  size_t smA = (size_t)std::max(epb, ka.epb_a) * ka.layA.team_doubles * 8,
         smB = (size_t)epb * ka.layB.team_doubles * 8;
  if ((e = sse_set_smem_limits(ka, smA, smB)) != cudaSuccess) return cuda_fail(s, e, "cudaFuncSetAttribute");

  // the weight-adjusted mass operator V' diag(J^-1 W) V of every element,
  // built once when it takes at most a quarter of the free device memory:
  // each mass solve is then one dense n_p x n_p product instead of two
  // sum-factorised applications of V
  ka.Ak = nullptr;
  if (has_vdm && c.mass_solver == SSE_WEIGHT_ADJUSTED) {
    const size_t bytes = (size_t)c.n_e * np * np * 8;
    size_t freeb = 0, totalb = 0;
    if ((e = cudaMemGetInfo(&freeb, &totalb))) return cuda_fail(s, e, "cudaMemGetInfo");
    if (bytes <= freeb / 4) {
      if ((e = alloc(s, bytes, &p))) return cuda_fail(s, e, "alloc mass operators");
      if ((e = launch_mass_operator(ka, (double *)p, s->stream))) return cuda_fail(s, e, "mass operators");
      if ((e = cudaStreamSynchronize(s->stream))) return cuda_fail(s, e, "mass operators");
      ka.Ak = (const double *)p;
    }
  }
  return setup_compact(s, ops, mapP);
}

// Reads the device flag into pinned host memory behind the stream's work:
// one synchronisation covers that work and the read.
int check_flag(sse_solver *s) {
  cudaError_t e = cudaMemcpyAsync(s->h_flag, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_fail(s, e, "flag read");
  const int h = *s->h_flag;
  if (h) {
    cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream);
    cudaStreamSynchronize(s->stream);
    if (h & 2) return fail(s, SSE_ERR_CUDA, "a kernel's bounded wait for its shared-memory copies gave up");
    return fail(s, SSE_ERR_NONPHYSICAL, "non-physical state (density/pressure <= 0 or non-finite residual)");
  }
  return SSE_OK;
}

// Mixed form: FP32 roundings of the metric terms and operator values, FP32
// perturbation scratch, FP64 compensation buffer.  Allocated once.
int enable_mixed(sse_solver *s) {
  const sse_config &c = s->cfg;
  if (!(c.form == SSE_FLUX_DIFFERENCING_FORM && c.law == SSE_EULER && c.two_point_flux == SSE_EC_FLUX))
    return fail(s, SSE_ERR_UNSUPPORTED,
                "SSE_MIXED covers FluxDifferencingForm with the entropy-conservative flux (Euler)");
  if (s->ka.op.has_vdm && s->mode0 < 0)
    return fail(s, SSE_ERR_UNSUPPORTED, "SSE_MIXED needs a modal basis with a constant basis function");
  if (s->mixed_ready) return SSE_OK;
  KernelArgs &ka = s->ka;
  DevOps &op = ka.op;
  DevGeo &g = ka.geo;
  cudaError_t e;
  void *p;
  auto rounded = [&](const double *src, size_t n, const float **dst) -> cudaError_t {
    *dst = nullptr;
    if (!src || n == 0) return cudaSuccess;
    void *q = nullptr;
    cudaError_t err = alloc(s, n * sizeof(float), &q);
    if (err != cudaSuccess) return err;
    *dst = (const float *)q;
    return launch_round_to_float(src, (float *)q, n, s->stream);
  };
  const size_t nq = c.n_q, nf = c.n_f, ne = c.n_e, d = c.d;
  if ((e = rounded(op.A, s->nA, &op.Af)) || (e = rounded(op.B, s->nB, &op.Bf)) ||
      (e = rounded(op.C, s->nC, &op.Cf)) || (e = rounded(op.R_val, s->nnzR, &op.R_valf)) ||
      (e = rounded(op.Rt_val, s->nnzR, &op.Rt_valf)) || (e = rounded(op.vp_S, s->nvpS, &op.vp_Sf)) ||
      (e = rounded(op.fp_C, s->nfpC, &op.fp_Cf)) || (e = rounded(op.Vd, s->nVd, &op.Vdf)))
    return cuda_fail(s, e, "mixed operators");
  op.vp_pkf = op.fp_pkf = nullptr;
  if (op.nvp + op.nfp > 0) {
    void *pv = nullptr, *pf = nullptr;
    if ((e = alloc(s, (size_t)std::max(op.nvp, 1) * 4 * sizeof(float), &pv)) ||
        (e = alloc(s, (size_t)std::max(op.nfp, 1) * 2 * sizeof(float), &pf)) ||
        (e = launch_pack_pairs(op, (float *)pv, (float *)pf, s->stream)))
      return cuda_fail(s, e, "mixed pair tables");
    op.vp_pkf = (const float *)pv;
    op.fp_pkf = (const float *)pf;
  }
  // the per-element mass operators in FP32, transposed to row-major (the FP32
  // dense solve gives each thread one row)
  ka.Akf = nullptr;
  if (ka.Ak) {
    if ((e = alloc(s, (size_t)c.n_e * c.n_p * c.n_p * sizeof(float), &p)) ||
        (e = launch_round_transpose(ka.Ak, (float *)p, c.n_e, c.n_p, s->stream)))
      return cuda_fail(s, e, "mixed mass operators");
    ka.Akf = (const float *)p;
  }
  g.halfnJqt = nullptr;
  if (g.halfnJq) {
    if ((e = alloc(s, (size_t)d * c.num_faces * nq * ne * sizeof(float), &p)) ||
        (e = launch_halfnjq_transpose(g.halfnJq, (float *)p, ne, (int)nq, (int)d, c.num_faces, s->stream)))
      return cuda_fail(s, e, "mixed metric terms");
    g.halfnJqt = (const float *)p;
  }
  g.Lambda_qn = nullptr;
  if (g.Lambda_q) {
    if ((e = alloc(s, (size_t)lambda_stride((int)d) * nq * ne * sizeof(float), &p)) ||
        (e = launch_lambda_node_major(g.Lambda_q, (float *)p, ne, (int)nq, (int)d, s->stream)))
      return cuda_fail(s, e, "mixed metric terms");
    g.Lambda_qn = (const float *)p;
  }
  if ((e = rounded(g.BJf, nf * ne, &g.BJff)) || (e = rounded(g.n_f, d * nf * ne, &g.n_ff)) ||
      (e = rounded(g.halfnJf, d * nf * ne, &g.halfnJff)) ||
      (e = rounded(g.halfnJq, d * c.num_faces * nq * ne, &g.halfnJqf)) ||
      (e = rounded(g.JinvW, g.JinvW ? nq * ne : 0, &g.JinvWf)) ||
      (e = rounded(g.WJinv, g.WJinv ? nq * ne : 0, &g.WJinvf)))
    return cuda_fail(s, e, "mixed metric terms");
  if ((e = alloc(s, nq * c.n_c * ne * sizeof(float), &p))) return cuda_fail(s, e, "alloc");
  ka.u_qf = (float *)p;
  if ((e = alloc(s, nf * c.n_c * ne * sizeof(float), &p))) return cuda_fail(s, e, "alloc");
  ka.u_ff = (float *)p;
  if ((e = alloc(s, (size_t)c.n_p * c.n_c * ne * sizeof(double), &p))) return cuda_fail(s, e, "alloc");
  s->d_comp = (double *)p;
  // the reference state's FP64 residual (filled when the state is chosen)
  // and the host buffer of the reduction that chooses it: allocated here so
  // that no later call allocates
  if ((e = alloc(s, (size_t)c.n_p * c.n_c * ne * sizeof(double), &p))) return cuda_fail(s, e, "alloc");
  s->d_rref = (double *)p;
  s->h_partial.assign((size_t)c.n_e * (c.n_c + 1), 0.0);
  // phase-B layout in floats (primitives carry p - p_ref as well)
  const int nc = c.n_c, np = c.n_p;
  int zsz = 0, wsz = 0;
  if (op.has_vdm) {
    if (c.d == 2) zsz = nc * op.p1 * op.M2;
    else { zsz = nc * op.nb12 * op.M3; wsz = nc * op.p1 * op.M2 * op.M3; }
  }
  // the pair buffer holds one chunk of pair contributions, then the modal /
  // nodal buffers and the sum-factorisation scratch of the lift; all pairs
  // at once when four blocks fit on an SM, else chunks (a whole number of
  // passes of the element's threads) that keep four
  auto r4 = [](int n) { return (n + 3) & ~3; };
  const int zsz4 = r4(zsz);
  const int final_m = nc * (np + (int)nq) + zsz4 + wsz;
  const int max_pairs = std::max(op.nvp, op.nfp);
  // phase B in FP32 keeps teams of at least 32 threads in blocks of the same
  // size (16-thread teams made the 2-D vortex's phase B 39 % slower: it is
  // latency-bound, and narrower teams lengthen each element's chains)
  const int tpe_fp64 = ka.tpb / ka.epb;
  const int tpe_m = std::max(32, tpe_fp64);
  ka.epb_bm = std::max(1, ka.epb * tpe_fp64 / tpe_m);
  // Shared regions of the staged slabs: n floats plus the alignment margin
  // of a bulk copy (the slab lands at its source address modulo 16).
  auto staged = [&](int n) { return r4(n + 8); };
  const int quads = (int)((nq + nf + 3) / 4);
  // phase-B layout, pair chunk and optional staged slabs for the
  // sum-factorised tail (et = false) or the tail operators (et = true: region
  // 2 holds the node-major residuals, 8 floats per node with the last column
  // quad's padding nodes, and the pair buffer later the G = tpe / n_p partial
  // rows of the tail product)
  struct Plan { int chunk, blocks, off; bool geo, rref, ak; };
  auto plan = [&](bool et) {
    const int np2 = ka.Akf && !et ? np * np : 0;
    const int region2 = et ? (nc > 4 ? 20 : 16) * quads : nc * (int)nf;  // quads of node-major residuals
    const int final_e = et ? (tpe_m / np) * np * 8 : final_m;
    auto layout_m = [&](int chunk, bool geo, bool rref, bool ak) {
      const int sizes[11] = {staged(nc * (int)nq), staged(nc * (int)nf), region2,
                             ak && np2 ? staged(np2) : 0, std::max(chunk * nc, final_e),
                             staged(lambda_stride((int)d) * (int)nq), op.nfp > 0 ? staged((int)(d * c.num_faces * nq)) : 0,
                             (int)((nq + nf) * (4 + d)),
                             geo ? 2 * staged((int)(d * nf)) + staged((int)nf) : 0,
                             rref ? staged(2 * nc * np) : 0, 4};
      int off = 0, i = 0;
      for (int sz : sizes) { ka.layBm.off[i++] = off; off += r4(sz); }
      for (; i < 12; ++i) ka.layBm.off[i] = off;
      ka.layBm.team_doubles = off;  // counted in floats for this layout
      return off;
    };
    const int budget_m = (int)((size_t)55 * 1024 / 4 / ka.epb_bm);
    int chunk_m = max_pairs;
    if (layout_m(chunk_m, false, false, false) > budget_m) {
      // four blocks per SM when chunks of at least one pass of the element's
      // threads fit, else two, else one
      const int fixed = layout_m(0, false, false, false) - r4(final_e);
      const int need = std::min(tpe_m, max_pairs) * nc;
      int room = budget_m - fixed;
      if (room < need) room = 2 * budget_m - fixed;
      if (room < need) room = (int)((size_t)220 * 1024 / 4 / ka.epb_bm) - fixed;
      chunk_m = std::max(1, room / nc);
      if (chunk_m >= tpe_m) chunk_m = chunk_m / tpe_m * tpe_m;
      chunk_m = std::max(1, std::min(chunk_m, max_pairs));
    }
    // The facet geometry, the reference residual and the mass operator are
    // staged as well where that keeps the resident blocks per SM (shared
    // memory, registers and threads together), else read from global memory.
    auto blocks_per_sm = [&](int floats) {
      int nb = 0;
      if (sse_mixed_b_blocks_per_sm(ka, (size_t)ka.epb_bm * floats * 4, &nb) != cudaSuccess) return 0;
      return nb;
    };
    Plan pl{chunk_m, 0, 0, false, false, false};
    pl.blocks = blocks_per_sm(layout_m(chunk_m, false, false, false));
    if (blocks_per_sm(layout_m(chunk_m, true, false, false)) >= pl.blocks) pl.geo = true;
    if (blocks_per_sm(layout_m(chunk_m, pl.geo, true, false)) >= pl.blocks) pl.rref = true;
    if (blocks_per_sm(layout_m(chunk_m, pl.geo, pl.rref, true)) >= pl.blocks) pl.ak = true;
    pl.off = layout_m(chunk_m, pl.geo, pl.rref, pl.ak);
    return pl;
  };
  // The tail operators E_k = A_k V^T [I | -R^T]: phase B's lift, V^T and
  // weight-adjusted mass solve as one per-element product, built once in
  // FP64 and rounded to FP32, where the FP64 mass operators exist, the
  // element's threads cover its n_p rows, the operators take at most a
  // quarter of the free device memory, and the node-major residuals keep
  // the blocks per SM and the pair chunk of the sum-factorised tail (p = 5
  // tets: the tail operators cost a smaller chunk, and phase B took 10.7
  // instead of 5.3 ms).
  ka.Ekf = nullptr;
  ka.ek_quads = 0;
  Plan chosen = plan(false);
  if (ka.Ak && ka.Akf && op.has_vdm && tpe_m >= np) {
    const size_t bytes = (size_t)ne * quads * np * 16;
    size_t freeb = 0, totalb = 0;
    if ((e = cudaMemGetInfo(&freeb, &totalb))) return cuda_fail(s, e, "cudaMemGetInfo");
    ka.Ekf = reinterpret_cast<const float *>(16);  // selects the instantiation for the occupancy query
    ka.ek_quads = quads;
    const Plan withE = plan(true);
    ka.Ekf = nullptr;
    ka.ek_quads = 0;
    if (bytes <= freeb / 4 && withE.chunk >= chosen.chunk && withE.blocks >= chosen.blocks) {
      const double *Vd = op.dense_v ? op.Vd : nullptr;
      if (!Vd) {
        if ((e = alloc(s, nq * np * sizeof(double), &p))) return cuda_fail(s, e, "alloc dense V");
        if ((e = launch_dense_vdm(ka, (double *)p, s->stream))) return cuda_fail(s, e, "dense V");
        Vd = (const double *)p;
      }
      void *pm = nullptr, *pe = nullptr;
      if ((e = alloc(s, (size_t)np * 4 * quads * sizeof(double), &pm)) || (e = alloc(s, bytes, &pe)) ||
          (e = launch_tail_operators(ka, Vd, (double *)pm, (float *)pe, quads, s->stream)))
        return cuda_fail(s, e, "mixed tail operators");
      ka.Ekf = (const float *)pe;
      ka.ek_quads = quads;
      chosen = plan(true);
    } else {
      chosen = plan(false);  // restores the layout of the sum-factorised tail
    }
  }
  ka.fd_chunk_mixed = chosen.chunk;
  ka.vdm_zsz_mixed = zsz4;
  const int off = chosen.off;
  size_t smm = (size_t)ka.epb_bm * off * sizeof(float);
  if (smm > 220 * 1024) return fail(s, SSE_ERR_UNSUPPORTED, "element too large for the mixed kernel");
  if ((e = sse_set_smem_limit_mixed(ka, smm))) return cuda_fail(s, e, "cudaFuncSetAttribute");
  if (op.has_vdm) {
    // phase A with FP32 projection arithmetic: layouts, and the FP64
    // projection of the constant function on every element
    auto ev = [](int n) { return (n + 1) & ~1; };
    const int big = nc * std::max(np, (int)nq), bigf = nc * std::max({np, (int)nq, (int)nf});
    Layout &A = ka.layAm;
    for (int i = 0; i < 5; ++i) A.off[i] = 0;      // no FP64 arrays: the float region starts at 0
    A.off[5] = 0;                                  // floats from here on
    A.off[6] = A.off[5] + ev(bigf);
    A.off[7] = A.off[6] + ev(nc * (int)nq);
    A.off[8] = A.off[7] + ev(big);
    A.off[9] = A.off[8] + ev(zsz);
    const int nfloats = A.off[9] + ev(wsz);
    for (int i = 10; i < 12; ++i) A.off[i] = 0;
    A.team_doubles = A.off[4] + nfloats / 2;
    // the FP32 phase A (barrier- and issue-bound) on 128-thread teams, two
    // elements per block, where the FP64 form uses 256 threads and the
    // element's volume and facet nodes fit in two passes of 128 (p = 4 tets:
    // 0.525 -> 0.400 ms per stage; p = 5 unchanged, p = 6 0.57 -> 0.72 ms)
    ka.epb_am = (tpe_fp64 >= 256 && nq + nf <= 256) ? ka.epb * (tpe_fp64 / 128) : ka.epb;
    int zsz1 = 0, wsz1 = 0;
    if (c.d == 2) zsz1 = op.p1 * op.M2;
    else { zsz1 = op.nb12 * op.M3; wsz1 = op.p1 * op.M2 * op.M3; }
    Layout &P = ka.layP1;
    const int big1 = std::max({np, (int)nq, (int)nf});
    const int sizes1[5] = {big1, (int)nq, zsz1, wsz1, big1};
    int o1 = 0;
    for (int i = 0; i < 5; ++i) { P.off[i] = o1; o1 += ev(sizes1[i]); }
    for (int i = 5; i < 12; ++i) P.off[i] = o1;
    P.team_doubles = o1;
    if ((size_t)std::max(ka.epb_am * A.team_doubles, ka.epb * P.team_doubles) * 8 > 220 * 1024)
      return fail(s, SSE_ERR_UNSUPPORTED, "element too large for the mixed projection kernel");
    if ((e = sse_set_smem_limits_mixed_a(ka))) return cuda_fail(s, e, "cudaFuncSetAttribute");
    if ((e = alloc(s, nq * ne * sizeof(double), &p))) return cuda_fail(s, e, "alloc");
    double *P1 = (double *)p;
    if ((e = alloc(s, nf * ne * sizeof(double), &p))) return cuda_fail(s, e, "alloc");
    double *RP1 = (double *)p;
    if ((e = launch_projection_of_one(ka, P1, RP1, s->stream))) return cuda_fail(s, e, "projection of 1");
    g.P1 = P1;
    g.RP1 = RP1;
    void *q1, *q2, *q3;
    if ((e = alloc(s, nq * ne * sizeof(float), &q1)) || (e = alloc(s, nf * ne * sizeof(float), &q2)) ||
        (e = alloc(s, nq * ne * sizeof(float), &q3)) ||
        (e = launch_round_to_float(P1, (float *)q1, nq * ne, s->stream, -1.0)) ||
        (e = launch_round_to_float(RP1, (float *)q2, nf * ne, s->stream, -1.0)) ||
        (e = launch_round_to_float(g.WJ, (float *)q3, nq * ne, s->stream)))
      return cuda_fail(s, e, "mixed projection constants");
    g.P1m1f = (const float *)q1;
    g.RP1m1f = (const float *)q2;
    g.WJf = (const float *)q3;
  }
  if ((e = cudaStreamSynchronize(s->stream))) return cuda_fail(s, e, "sync");
  s->mixed_ready = true;
  return SSE_OK;
}

// Choose the mixed form's reference state from the first state it sees:
// volume means of density and total energy, zero momentum.  Any constant
// state gives the same residual in exact arithmetic; a close one keeps the
// FP32 perturbations small.
int ensure_reference(sse_solver *s, const double *u_dev) {
  if (s->ref_ready) return SSE_OK;
  const sse_config &c = s->cfg;
  cudaError_t e = launch_conservation(s->ka, u_dev, u_dev, s->d_partial, s->stream);
  if (e != cudaSuccess) return cuda_fail(s, e, "reference state");
  std::vector<double> &part = s->h_partial;
  if ((e = cudaMemcpyAsync(part.data(), s->d_partial, part.size() * 8, cudaMemcpyDeviceToHost, s->stream)) ||
      (e = cudaStreamSynchronize(s->stream)))
    return cuda_fail(s, e, "reference state");
  double rho = 0.0, E = 0.0;
  for (int k = 0; k < c.n_e; ++k) {
    rho += part[(size_t)k * (c.n_c + 1)];
    E += part[(size_t)k * (c.n_c + 1) + c.n_c - 1];
  }
  Physics &ph = s->ka.ph;
  ph.rho_ref = rho / s->volume;
  ph.E_ref = E / s->volume;
  ph.p_ref = ph.gm1 * ph.E_ref;
  ph.theta_ref = ph.p_ref / ph.rho_ref;
  ph.H_ref = ph.gamma / ph.gm1 * ph.theta_ref;
  {
    double uref[5] = {ph.rho_ref, 0.0, 0.0, 0.0, 0.0};
    uref[c.n_c - 1] = ph.E_ref;
    if (c.d == 2) cons_to_entropy_fast<2>(ph.gamma, ph.gm1, ph.igm1, uref, ph.w_ref);
    else cons_to_entropy_fast<3>(ph.gamma, ph.gm1, ph.igm1, uref, ph.w_ref);
    // constants of the mixed-form entropy maps around the reference state
    ph.mode0 = s->mode0;
    for (int e = 0; e < 5; ++e) ph.u_ref_modal[e] = s->phi0 != 0.0 ? uref[e] / s->phi0 : 0.0;
    ph.ip_ref = 1.0 / ph.p_ref;
    ph.irho_ref = 1.0 / ph.rho_ref;
    ph.a_ref = -ph.gm1 * ph.w_ref[c.n_c - 1];
    ph.ia_ref = 1.0 / ph.a_ref;
    ph.rhoe_ref = ph.E_ref;  // internal energy p_ref / (gamma - 1) at zero velocity
  }
  if (!(ph.rho_ref > 0.0) || !(ph.p_ref > 0.0))
    return fail(s, SSE_ERR_NONPHYSICAL, "mixed form: mean density or energy not positive");
  ph.f_gamma = (float)ph.gamma;
  ph.f_gm1 = (float)ph.gm1;
  ph.f_igm1 = (float)ph.igm1;
  ph.f_half_lambda = (float)ph.half_lambda;
  ph.f_rho_ref = (float)ph.rho_ref;
  ph.f_p_ref = (float)ph.p_ref;
  ph.f_theta_ref = (float)ph.theta_ref;
  ph.f_H_ref = (float)ph.H_ref;
  ph.f_E_ref = (float)ph.E_ref;
  ph.cref = entropy_ref_f(ph);
  // The FP32 phase B leaves the reference pressure out of every momentum
  // flux; those terms are the FP64 phase-B residual of u_ref at its nodal
  // states.  Evaluate it once (FP64 phase B on constant nodal scratch) for
  // the mixed phase B to add back: on metrics that do not preserve a free
  // stream (exact metrics on curved tets) it is O(p_ref), not round-off.
  {
    double uref[5] = {ph.rho_ref, 0.0, 0.0, 0.0, 0.0};
    uref[c.n_c - 1] = ph.E_ref;
    KernelArgs kb = s->ka;
    kb.mixed = 0;
    kb.dudt = s->d_rref;
    if ((e = launch_fill_constant_state(kb.u_q, c.n_q, c.n_c, c.n_e, uref, s->stream)) ||
        (e = launch_fill_constant_state(kb.u_f, c.n_f, c.n_c, c.n_e, uref, s->stream)) ||
        (e = launch_time_derivative(kb, s->stream)) || (e = cudaStreamSynchronize(s->stream)))
      return cuda_fail(s, e, "reference-state residual");
    s->ka.geo.Rref = s->d_rref;
  }
  s->ref_ready = true;
  return SSE_OK;
}

// one residual evaluation on device buffers (no synchronisation in the FP64
// form; the mixed form synchronises once, on its first call).  u_q / u_f,
// when given, receive the FP64 nodal states instead of the handle's scratch.
// The one-kernel StandardForm path runs unless nodal states are asked for or
// two_phase is set.
cudaError_t residual_device(sse_solver *s, const double *u, double *dudt, double *u_q = nullptr,
                            double *u_f = nullptr, bool two_phase = false) {
  if (s->ka.mixed && !s->ref_ready && ensure_reference(s, u) != SSE_OK) return cudaErrorInvalidValue;
  KernelArgs ka = s->ka;
  // (a residual written over its own input, which the neighbours' traces
  // read, takes the two-phase kernels)
  if (ka.compact && !u_q && !two_phase && dudt != u) {
    CompactStage st{};
    st.mode = kCompactResidual;
    st.uin = u;
    st.out = dudt;
    return launch_std_compact(ka, st, s->stream);
  }
  ka.u = u;
  ka.dudt = dudt;
  if (u_q) {
    ka.u_q = u_q;
    ka.u_f = u_f;
  }
  // NVTX ranges named like the reference's TimerOutputs sections
  // (Solvers.jl:474-489), around each phase's launch
  nvtxRangePushA("nodal values");
  cudaError_t e = launch_nodal_values(ka, s->stream);
  nvtxRangePop();
  if (e != cudaSuccess) return e;
  nvtxRangePushA("time deriv.");
  e = launch_time_derivative(ka, s->stream);
  nvtxRangePop();
  return e;
}

// ---------------------------------------------------------------------------
// Discrete adjoint
// ---------------------------------------------------------------------------

// VJP scratch and shared-memory layouts of the three adjoint kernels.
int enable_adjoint(sse_solver *s) {
  const sse_config &c = s->cfg;
  const bool fd = c.form == SSE_FLUX_DIFFERENCING_FORM;
  // FluxDifferencingForm pair transposes: the contracted entropy-conservative
  // flux (Euler) or the conservative two-point flux (advection, Euler with
  // ConservativeFlux)
  const bool ec_pairs = c.law == SSE_EULER && c.two_point_flux == SSE_EC_FLUX;
  if (fd && c.law == SSE_EULER && c.two_point_flux == SSE_CHANDRASHEKAR_FLUX)
    return fail(s, SSE_ERR_UNSUPPORTED, "the discrete adjoint does not cover Chandrashekar's two-point flux");
  if (!s->mapP_involution)
    return fail(s, SSE_ERR_UNSUPPORTED, "the discrete adjoint needs mapP to pair facet nodes (mapP(mapP(x)) == x)");
  if (s->adj_ready) return SSE_OK;
  KernelArgs &ka = s->ka;
  const DevOps &op = ka.op;
  const int nc = c.n_c, np = c.n_p, nq = c.n_q, nf = c.n_f, d = c.d, ps = 3 + d;
  int zsz = 0, wsz = 0;
  if (op.has_vdm) {
    if (d == 2) zsz = nc * op.p1 * op.M2;
    else { zsz = nc * op.nb12 * op.M3; wsz = nc * op.p1 * op.M2 * op.M3; }
  }
  auto finish = [](Layout &L, std::initializer_list<int> sizes) {
    int off = 0, i = 0;
    for (int sz : sizes) { L.off[i++] = off; off += (sz + 1) & ~1; }
    for (; i < 12; ++i) L.off[i] = off;
    L.team_doubles = off;
  };
  const size_t cap = (size_t)220 * 1024 / 8 / ka.epb;  // doubles per team
  const int tpe_adj = ka.tpb / ka.epb;
  // lift (and the plain nodal-values transpose): X, Y, Z, W, F as in phase A
  ka.layAdjB1 = ka.layA;
  cudaError_t e;
  void *p;
  const size_t ne = c.n_e, n = (size_t)np * nc * ne;
  auto alloc_vjp = [&]() -> int {
    if ((e = alloc(s, (size_t)nq * nc * ne * 8, &p))) return cuda_fail(s, e, "alloc"); ka.rbar_q = (double *)p;
    if ((e = alloc(s, (size_t)nf * nc * ne * 8, &p))) return cuda_fail(s, e, "alloc"); ka.gbar_f = (double *)p;
    if ((e = alloc(s, (size_t)nq * nc * ne * 8, &p))) return cuda_fail(s, e, "alloc"); ka.ubar_q = (double *)p;
    if ((e = alloc(s, (size_t)nf * nc * ne * 8, &p))) return cuda_fail(s, e, "alloc"); ka.ubar_f = (double *)p;
    if ((e = alloc(s, n * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_lam = (double *)p;
    if ((e = alloc(s, n * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_mu = (double *)p;
    if ((e = sse_set_smem_limits_adjoint(ka))) return cuda_fail(s, e, "cudaFuncSetAttribute (adjoint)");
    s->adj_ready = true;
    return SSE_OK;
  };
  if (!fd) {
    // StandardForm flux transposes: u_q, u_f, rbar_q, gbar_f, fbar_n (d of
    // them), two volume temporaries, one facet temporary
    finish(ka.layAdjS, {nc * nq, nc * nf, nc * nq, nc * nf, d * nc * nq, nc * nq, nc * nq, nc * nf});
    if (ka.layAdjS.team_doubles > (int)cap)
      return fail(s, SSE_ERR_UNSUPPORTED, "element too large for the adjoint kernels' shared memory");
    return alloc_vjp();
  }
  // projection transpose: X, Y, Z, W, F, u_q0, w_q, w_f, ubar_q, ubar_f
  finish(ka.layAdjA, {nc * std::max(np, nq), nc * nq, zsz, wsz, nc * std::max({np, nq, nf}), nc * nq,
                      nc * nq, nc * nf, nc * nq, nc * nf});
  if (ka.layAdjA.team_doubles > (int)cap)
    return fail(s, SSE_ERR_UNSUPPORTED, "element too large for the adjoint kernels' shared memory");
  const int hsz = op.nfp > 0 ? d * c.num_faces * nq : 0;
  const int max_pairs = std::max(op.nvp, op.nfp);
  if (!ec_pairs) {
    // conservative two-point flux: u_q, u_f, rbar_q, fbar_f, ubar_q, ubar_f,
    // Lambda_q, halfnJq, then a chunk of per-pair state cotangents (2 NC each)
    Layout gbase{};
    finish(gbase, {nc * nq, nc * nf, nc * nq, nc * nf, nc * nq, nc * nf, d * d * nq, hsz});
    long room = (long)(110 * 1024 / 8 / ka.epb) - gbase.team_doubles;
    if (room < 128 * 2 * nc) room = (long)cap - gbase.team_doubles;
    int chunk = (int)std::min<long>(max_pairs, room / (2 * nc));
    if (chunk >= tpe_adj) chunk = chunk / tpe_adj * tpe_adj;
    if (chunk < 1)
      return fail(s, SSE_ERR_UNSUPPORTED, "element too large for the adjoint kernels' shared memory");
    ka.pair_chunk_generic = chunk;
    finish(ka.layAdjG, {nc * nq, nc * nf, nc * nq, nc * nf, nc * nq, nc * nf, d * d * nq, hsz,
                        chunk * 2 * nc});
    return alloc_vjp();
  }
  // pair transposes: fixed arrays, then a chunk of per-pair primitive cotangents
  Layout base{};
  finish(base, {nc * nq, nc * nf, nc * nq, nc * nf, (nq + nf) * ps, (nq + nf) * ps, nc * nf, d * d * nq, hsz});
  // chunk: as large as keeps two blocks per SM when that leaves at least
  // 128 pairs; otherwise one block per SM with chunks as large as fit
  long room = (long)(110 * 1024 / 8 / ka.epb) - base.team_doubles;
  if (room < 128 * 2 * ps) room = (long)cap - base.team_doubles;
  int chunk = (int)std::min<long>(max_pairs, room / (2 * ps));
  if (chunk >= tpe_adj) chunk = chunk / tpe_adj * tpe_adj;
  if (chunk < 1)
    return fail(s, SSE_ERR_UNSUPPORTED, "element too large for the adjoint kernels' shared memory");
  ka.pair_chunk = chunk;
  finish(ka.layAdjB2, {nc * nq, nc * nf, nc * nq, nc * nf, (nq + nf) * ps, (nq + nf) * ps, nc * nf,
                       d * d * nq, hsz, chunk * 2 * ps});
  return alloc_vjp();
}

// Layouts (in floats) of the mixed-form VJP kernels; needs enable_adjoint
// and enable_mixed first.
int enable_adjoint_mixed(sse_solver *s) {
  if (s->adj_mixed_ready) return SSE_OK;
  const sse_config &c = s->cfg;
  KernelArgs &ka = s->ka;
  const DevOps &op = ka.op;
  if (!op.has_vdm)
    return fail(s, SSE_ERR_UNSUPPORTED, "the mixed-form adjoint covers modal (ModalTensor) bases");
  const int nc = c.n_c, np = c.n_p, nq = c.n_q, nf = c.n_f, d = c.d, ps = 4 + d;
  int zsz = 0, wsz = 0;
  if (d == 2) zsz = nc * op.p1 * op.M2;
  else { zsz = nc * op.nb12 * op.M3; wsz = nc * op.p1 * op.M2 * op.M3; }
  auto r4 = [](int n) { return (n + 3) & ~3; };
  auto finish = [&](Layout &L, std::initializer_list<int> sizes) {
    int off = 0, i = 0;
    for (int sz : sizes) { L.off[i++] = off; off += r4(sz); }
    for (; i < 12; ++i) L.off[i] = off;
    L.team_doubles = off;  // counted in floats for these layouts
  };
  const int big = nc * std::max(np, nq), bigf = nc * std::max({np, nq, nf});
  finish(ka.layAdjB1m, {big, nc * nq, zsz, wsz, bigf});
  finish(ka.layAdjAm, {big, nc * nq, nc * nq, nc * nq, nc * nf, big, nc * nq, zsz, wsz, nc * nf});
  int hsz = op.nfp > 0 ? d * c.num_faces * nq : 0;
  Layout base{};
  finish(base, {nc * nq, nc * nf, nc * nq, nc * nf, (nq + nf) * ps, (nq + nf) * ps, nc * nf, d * d * nq, hsz});
  const int max_pairs = std::max(op.nvp, op.nfp);
  const int tpe_adj = ka.tpb / ka.epb;
  const long cap = (long)(220 * 1024 / 4 / ka.epb);          // floats per team
  const long four = (long)(55 * 1024 / 4 / ka.epb);          // team size for four blocks per SM
  if (four - base.team_doubles < 128 * 2 * ps && four - (base.team_doubles - r4(hsz)) >= 128 * 2 * ps) {
    // halfnJq read from global memory keeps four blocks per SM
    hsz = 0;
    finish(base, {nc * nq, nc * nf, nc * nq, nc * nf, (nq + nf) * ps, (nq + nf) * ps, nc * nf, d * d * nq, 0});
  }
  long room = four - base.team_doubles;
  if (room < 128 * 2 * ps) room = (long)(110 * 1024 / 4 / ka.epb) - base.team_doubles;  // two
  if (room < 128 * 2 * ps) room = cap - base.team_doubles;
  int chunk = (int)std::min<long>(max_pairs, room / (2 * ps));
  if (chunk >= tpe_adj) chunk = chunk / tpe_adj * tpe_adj;
  if (chunk < 1 || (long)ka.layAdjAm.team_doubles > cap)
    return fail(s, SSE_ERR_UNSUPPORTED, "element too large for the mixed-form adjoint kernels");
  ka.pair_chunk_mixed = chunk;
  finish(ka.layAdjB2m, {nc * nq, nc * nf, nc * nq, nc * nf, (nq + nf) * ps, (nq + nf) * ps, nc * nf,
                        d * d * nq, hsz, chunk * 2 * ps});
  cudaError_t e;
  if ((e = sse_set_smem_limits_adjoint_mixed(ka))) return cuda_fail(s, e, "cudaFuncSetAttribute (mixed adjoint)");
  s->adj_mixed_ready = true;
  return SSE_OK;
}

// mu = (dR/du)^T lam for the mixed form at u: its phase A writes the FP32
// perturbation states, then the FP32 transposes run with lam~.
cudaError_t vjp_device_mixed(sse_solver *s, const double *u, const double *lam, double *mu) {
  KernelArgs ka = s->ka;
  ka.mixed = 1;
  ka.u = u;
  ka.lam = lam;
  ka.mu = mu;
  cudaError_t e = launch_nodal_values(ka, s->stream);
  if (e != cudaSuccess) return e;
  return launch_residual_vjp_mixed_kernels(ka, s->stream);
}

// mu = (dR/du)^T lam on device buffers.  u_q / u_f: the FP64 nodal states of
// u when already computed (a recorded stage), else phase A runs first.
cudaError_t vjp_device(sse_solver *s, const double *u, const double *lam, double *mu,
                       const double *u_q = nullptr, const double *u_f = nullptr) {
  KernelArgs ka = s->ka;
  ka.mixed = 0;
  ka.u = u;
  ka.lam = lam;
  ka.mu = mu;
  cudaError_t e;
  if (u_q) {
    ka.u_q = const_cast<double *>(u_q);
    ka.u_f = const_cast<double *>(u_f);
  } else if ((e = launch_nodal_values(ka, s->stream)) != cudaSuccess) {
    return e;
  }
  return launch_residual_vjp_kernels(ka, s->stream);
}

// one Runge-Kutta step of u (device) using the tape's work buffers; with
// slot >= 0 every stage's input state (and, for FP64 recordings, its nodal
// states) is stored in the segment slots slot*stages + stage
cudaError_t tape_step(sse_solver *s, double *u, int slot) {
  sse_solver::Tape &T = s->tape;
  const sse_config &c = s->cfg;
  const size_t n = (size_t)c.n_p * c.n_c * c.n_e;
  const size_t nqs = (size_t)c.n_q * c.n_c * c.n_e, nfs = (size_t)c.n_f * c.n_c * c.n_e;
  const double dt = T.dt;
  cudaError_t e;
  auto stage_residual = [&](const double *y, int st) -> cudaError_t {
    // the recording and every recomputation take the same two-phase kernels,
    // so each state of the trajectory is the same bits whichever produced it
    if (slot < 0) return residual_device(s, y, T.w_dudt, nullptr, nullptr, true);
    const size_t q = (size_t)slot * T.stages + st;
    double *ys = T.seg_y + q * n;
    cudaError_t err = cudaMemcpyAsync(ys, y, n * 8, cudaMemcpyDeviceToDevice, s->stream);
    if (err != cudaSuccess) return err;
    if (T.nodal) return residual_device(s, ys, T.w_dudt, T.seg_uq + q * nqs, T.seg_uf + q * nfs);
    return residual_device(s, ys, T.w_dudt, nullptr, nullptr, true);
  };
  if (T.scheme == SSE_CARPENTER_KENNEDY_2N54) {
    for (int st = 0; st < 5; ++st) {
      if ((e = stage_residual(u, st))) return e;
      e = T.mixed ? launch_ck_stage_compensated(u, T.w_comp, T.w_tmp, T.w_dudt, kCKA[st], kCKB[st], dt,
                                                st == 0, n, s->stream)
                  : launch_ck_stage(u, T.w_tmp, T.w_dudt, kCKA[st], kCKB[st], dt, st == 0, n, s->stream);
      if (e) return e;
    }
    return cudaSuccess;
  }
  const double half = dt / 2;
  if ((e = stage_residual(u, 0))) return e;
  if ((e = launch_rk4_stage(u, T.w_ust, T.w_acc, T.w_dudt, 0.0, half, 1, n, s->stream))) return e;
  if ((e = stage_residual(T.w_ust, 1))) return e;
  if ((e = launch_rk4_stage(u, T.w_ust, T.w_acc, T.w_dudt, 2.0, half, 0, n, s->stream))) return e;
  if ((e = stage_residual(T.w_ust, 2))) return e;
  if ((e = launch_rk4_stage(u, T.w_ust, T.w_acc, T.w_dudt, 2.0, dt, 0, n, s->stream))) return e;
  if ((e = stage_residual(T.w_ust, 3))) return e;
  return launch_rk4_final(u, T.w_acc, T.w_dudt, dt / 6, n, s->stream);
}

// ---------------------------------------------------------------------------
// Binomial checkpointing of the Runge-Kutta trajectory (Griewank, Optim.
// Methods Softw. 1 (1992) 35-54; Griewank & Walther, ACM TOMS 26 (2000)
// 19-45, "revolve").  F(n, c) is the fewest extra forward steps that
// reverse n steps, the state before the first being held, with c free
// checkpoint slots:
//   F(1, c) = 0,  F(n, 0) = n (n - 1) / 2,
//   F(n, c) = min over 1 <= m < n of  m + F(n - m, c - 1) + F(m, c)
// (advance m steps, keep that state in a free slot, reverse the last n - m
// steps with one slot fewer, then the first m with all of them).  The table
// holds the optimum and its split m for n up to kBinomialMaxDP steps (fewer
// when many checkpoints would make it costlier than about 2e8 operations);
// longer horizons are halved until they reach it.
// ---------------------------------------------------------------------------
constexpr int kBinomialMaxDP = 2048;

struct BinomialTable {
  int N = 0, C = 0;
  std::vector<long long> F;
  std::vector<int> M;
  long long &f(int n, int c) { return F[(size_t)n * (C + 1) + c]; }
  int &m(int n, int c) { return M[(size_t)n * (C + 1) + c]; }
  void build(int n_max, int c_max) {
    // the table costs about N^2 C operations: at most 2e8 (more than N - 1
    // checkpoints never help for N steps)
    N = std::min(n_max, kBinomialMaxDP);
    while (N > 1 && (double)N * N * (std::min(c_max, N - 1) + 1) > 2e8) N = N * 3 / 4;
    C = std::max(0, std::min(c_max, N - 1));
    F.assign((size_t)(N + 1) * (C + 1), 0);
    M.assign((size_t)(N + 1) * (C + 1), 0);
    for (int n = 1; n <= N; ++n)
      for (int c = 0; c <= C; ++c) {
        if (n == 1) { f(n, c) = 0; m(n, c) = 0; continue; }
        if (c == 0) { f(n, c) = (long long)n * (n - 1) / 2; m(n, c) = 0; continue; }
        long long best = -1;
        int arg = 1;
        for (int k = 1; k < n; ++k) {
          const long long v = k + f(n - k, c - 1) + f(k, c);
          if (best < 0 || v < best) { best = v; arg = k; }
        }
        f(n, c) = best;
        m(n, c) = arg;
      }
  }
  // with a slot for every step the optimum keeps every state (split 1)
  int split(int n, int c) { return c >= n - 1 ? 1 : (n <= N ? m(n, std::min(c, C)) : n / 2); }
};

enum : int { kActLoad = 0, kActAdvance = 1, kActStore = 2, kActRecRev = 3 };
inline int act(int kind, int arg) { return kind << 28 | arg; }
inline int act_kind(int a) { return a >> 28; }
inline int act_arg(int a) { return a & ((1 << 28) - 1); }

// The actions that reverse steps [l, r) with the state at l in slot sl and
// slots sl+1 .. sl+c free; returns the forward steps they evaluate.
long long binomial_plan(int l, int r, int c, int sl, BinomialTable &tab, std::vector<int> &out) {
  if (r - l == 1) {
    out.push_back(act(kActLoad, sl));
    out.push_back(act(kActRecRev, l));
    return 1;
  }
  if (c == 0) {
    long long steps = 0;
    for (int i = r - 1; i >= l; --i) {
      out.push_back(act(kActLoad, sl));
      if (i > l) out.push_back(act(kActAdvance, i - l));
      out.push_back(act(kActRecRev, i));
      steps += i - l + 1;
    }
    return steps;
  }
  const int m = l + tab.split(r - l, c);
  out.push_back(act(kActLoad, sl));
  out.push_back(act(kActAdvance, m - l));
  out.push_back(act(kActStore, sl + 1));
  long long steps = m - l;
  steps += binomial_plan(m, r, c - 1, sl + 1, tab, out);
  steps += binomial_plan(l, m, c, sl, tab, out);
  return steps;
}

// ---------------------------------------------------------------------------
// Fixed device scratch for sse_residual_static_scratch.
//
// The residual's two phases hand the element's volume and facet nodal states
// (u_q, u_f) from one kernel to the next through global memory.  For callers
// that must not allocate, that hand-over buffer is this file-scope array,
// present on every GPU that loads the library for the life of the process.
// Host code cannot use the symbol as a pointer: its device address is looked
// up with cudaGetSymbolAddress once per device, with that device current.
// ---------------------------------------------------------------------------
constexpr size_t kStaticScratchDoubles = SSE_STATIC_SCRATCH_BYTES / sizeof(double);
static __device__ __align__(256) double g_static_scratch[kStaticScratchDoubles];

constexpr int kMaxDevices = 64;
std::mutex g_static_scratch_mutex;
double *g_static_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (looked up on
// the first call per device).
int static_scratch_address(sse_solver *s, double **out) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_fail(s, e, "cudaGetDevice");
  if (dev < 0 || dev >= kMaxDevices) return fail(s, SSE_ERR_UNSUPPORTED, "device ordinal too large");
  std::lock_guard<std::mutex> lock(g_static_scratch_mutex);
  if (!g_static_scratch_addr[dev]) {
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess) return cuda_fail(s, e, "cudaGetSymbolAddress(static scratch)");
    g_static_scratch_addr[dev] = (double *)p;
  }
  *out = g_static_scratch_addr[dev];
  return SSE_OK;
}

}  // namespace

extern "C" {

int32_t sse_abi_version(void) { return SSE_ABI_VERSION; }

const char *sse_create_error(void) { return g_create_error.c_str(); }

const char *sse_last_error(const sse_solver *s) { return s ? s->last_error.c_str() : "null handle"; }

int32_t sse_create(const sse_config *cfg, const sse_operators *ops, const sse_geometry *geo,
                   sse_solver **out) {
  g_create_error.clear();
  if (!out) return fail(nullptr, SSE_ERR_INVALID_ARGUMENT, "out is null");
  *out = nullptr;
  if (!cfg || !ops || !geo) return fail(nullptr, SSE_ERR_INVALID_ARGUMENT, "null config/operators/geometry");
  sse_solver *s = nullptr;
  try {
    s = new sse_solver();
  } catch (const std::bad_alloc &) {
    return fail(nullptr, SSE_ERR_OUT_OF_MEMORY, "host allocation failed");
  }
  int rc;
  try {
    rc = build(s, cfg, ops, geo);
  } catch (const std::exception &ex) {
    rc = fail(s, SSE_ERR_OUT_OF_MEMORY, ex.what());
  }
  if (rc != SSE_OK) {
    g_create_error = s->last_error;
    sse_destroy(s);
    return rc;
  }
  *out = s;
  return SSE_OK;
}

int32_t sse_destroy(sse_solver *s) {
  if (!s) return SSE_OK;
  if (s->stream) cudaStreamSynchronize(s->stream);
  if (s->tape.block) cudaFree(s->tape.block);
  if (s->step_graph.exec) cudaGraphExecDestroy(s->step_graph.exec);
  for (void *p : s->allocations) cudaFree(p);
  if (s->h_flag) cudaFreeHost(s->h_flag);
  if (s->own_stream && s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return SSE_OK;
}

int32_t sse_set_stream(sse_solver *s, void *stream) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  cudaError_t e = cudaStreamSynchronize(s->stream);
  if (e != cudaSuccess) return cuda_fail(s, e, "sync");
  if (s->own_stream) cudaStreamDestroy(s->stream);
  s->own_stream = false;
  s->stream = (cudaStream_t)stream;
  return SSE_OK;
}

int32_t sse_set_precision(sse_solver *s, int32_t precision) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (precision == SSE_FP64) {
    s->ka.mixed = 0;
  } else if (precision == SSE_MIXED) {
    int rc = enable_mixed(s);
    if (rc != SSE_OK) return rc;
    s->ka.mixed = 1;
  } else {
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "precision must be SSE_FP64 or SSE_MIXED");
  }
  s->precision = precision;
  return SSE_OK;
}

// The device address of a host buffer of `bytes` bytes that kernels can reach
// in place: page-locked host memory mapped into the device's address space
// (cudaHostAlloc, or cudaHostRegister with mapping), first and last byte in
// the same mapping; null for pageable or unknown memory.
const void *mapped_host(const void *p, size_t bytes) {
  cudaPointerAttributes a{}, z{};
  const char *last = static_cast<const char *>(p) + (bytes ? bytes - 1 : 0);
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess || cudaPointerGetAttributes(&z, last) != cudaSuccess) {
    cudaGetLastError();  // clear the query's error for unknown (pageable) pointers
    return nullptr;
  }
  if (a.type != cudaMemoryTypeHost || z.type != cudaMemoryTypeHost || !a.devicePointer || !z.devicePointer)
    return nullptr;
  if (static_cast<const char *>(z.devicePointer) - static_cast<const char *>(a.devicePointer) !=
      last - static_cast<const char *>(p))
    return nullptr;
  return a.devicePointer;
}

int32_t sse_residual(sse_solver *s, const double *u, double *dudt, double t, int32_t memory) {
  (void)t;  // the supported laws carry no source term
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (!u || !dudt) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null u/dudt");
  size_t n = (size_t)s->cfg.n_p * s->cfg.n_c * s->cfg.n_e;
  cudaError_t e;
  if (memory == SSE_DEVICE) {
    if ((e = residual_device(s, u, dudt)) != cudaSuccess) return cuda_fail(s, e, "residual");
  } else if (memory == SSE_HOST) {
    const double *hu = static_cast<const double *>(mapped_host(u, n * 8));
    double *hd = static_cast<double *>(const_cast<void *>(mapped_host(dudt, n * 8)));
    if (hu && hd) {
      // page-locked caller buffers: phase A reads the state and phase B
      // writes the residual across the host link while they compute (GB300:
      // NVLink-C2C, ~190 GB/s either way, the rate of the staging copies),
      // so no copy stands between the stages
      if ((e = residual_device(s, hu, hd)) != cudaSuccess) return cuda_fail(s, e, "residual");
    } else {
      if ((e = cudaMemcpyAsync(s->d_u, u, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
      if ((e = residual_device(s, s->d_u, s->d_dudt)) != cudaSuccess) return cuda_fail(s, e, "residual");
      if ((e = cudaMemcpyAsync(dudt, s->d_dudt, n * 8, cudaMemcpyDeviceToHost, s->stream))) return cuda_fail(s, e, "D2H");
    }
  } else {
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "memory must be SSE_HOST or SSE_DEVICE");
  }
  return check_flag(s);
}

int32_t sse_residual_static_scratch(sse_solver *s, const double *u_dev, double *dudt_dev) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (!u_dev || !dudt_dev) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null u/dudt");
  if (s->ka.compact && dudt_dev != u_dev) {
    // the one-kernel StandardForm path keeps no nodal states at all
    CompactStage st{};
    st.mode = kCompactResidual;
    st.uin = u_dev;
    st.out = dudt_dev;
    cudaError_t e = launch_std_compact(s->ka, st, s->stream);
    if (e != cudaSuccess) return cuda_fail(s, e, "residual (static scratch)");
    return check_flag(s);
  }
  const sse_config &c = s->cfg;
  // the handle's precision: FP64 nodal states in the FP64 form, FP32
  // perturbation states in the mixed form (half the bytes per node)
  const bool mixed = s->ka.mixed != 0;
  const size_t word = mixed ? sizeof(float) : sizeof(double);
  const size_t nq = (size_t)c.n_q * c.n_c * c.n_e, nf = (size_t)c.n_f * c.n_c * c.n_e;
  // the mixed phase B stages each element's states with bulk copies of
  // their 16-byte-aligned spans, which may reach 15 bytes past the last one
  const size_t slack = mixed ? 64 : 0;
  if ((nq + nf) * word + slack > SSE_STATIC_SCRATCH_BYTES)
    return fail(s, SSE_ERR_INVALID_ARGUMENT,
                "mesh too large for the static scratch: needs " + std::to_string((nq + nf) * word) +
                    " bytes of nodal states, the fixed buffer holds " +
                    std::to_string((size_t)SSE_STATIC_SCRATCH_BYTES) + " (use sse_residual)");
  double *scratch = nullptr;
  int rc = static_scratch_address(s, &scratch);
  if (rc != SSE_OK) return rc;
  // the mixed form picks its reference state on its first call; that uses
  // buffers the handle allocated when SSE_MIXED was set, and synchronises
  if (mixed && (rc = ensure_reference(s, u_dev)) != SSE_OK) return rc;
  KernelArgs ka = s->ka;
  ka.u = u_dev;
  ka.dudt = dudt_dev;
  // the nodal states are fully written by phase A before phase B reads
  // them: no clearing needed between calls
  if (mixed) {
    ka.u_qf = reinterpret_cast<float *>(scratch);
    ka.u_ff = ka.u_qf + nq;
  } else {
    ka.u_q = scratch;
    ka.u_f = scratch + nq;
  }
  cudaError_t e = launch_nodal_values(ka, s->stream);
  if (e == cudaSuccess) e = launch_time_derivative(ka, s->stream);
  if (e != cudaSuccess) return cuda_fail(s, e, "residual (static scratch)");
  return check_flag(s);
}

int32_t sse_nodal_values(sse_solver *s, const double *u, double *u_q, double *u_f, int32_t memory) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (!u) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null u");
  const sse_config &c = s->cfg;
  size_t n = (size_t)c.n_p * c.n_c * c.n_e, nq = (size_t)c.n_q * c.n_c * c.n_e, nf = (size_t)c.n_f * c.n_c * c.n_e;
  cudaError_t e;
  const double *du = u;
  if (memory == SSE_HOST) {
    if ((e = cudaMemcpyAsync(s->d_u, u, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
    du = s->d_u;
  } else if (memory != SSE_DEVICE) {
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "memory must be SSE_HOST or SSE_DEVICE");
  }
  KernelArgs ka = s->ka;
  ka.mixed = 0;  // FP64 nodal values in the reference's layouts
  ka.u = du;
  if ((e = launch_nodal_values(ka, s->stream))) return cuda_fail(s, e, "nodal values");
  if (!s->d_uf_ref) {
    void *p;
    if ((e = alloc(s, nf * 8, &p))) return cuda_fail(s, e, "alloc");
    s->d_uf_ref = (double *)p;
  }
  if ((e = launch_facet_layout(ka.u_f, s->d_uf_ref, c.n_f, c.n_e, c.n_c, s->stream))) return cuda_fail(s, e, "layout");
  cudaMemcpyKind kind = memory == SSE_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if (u_q && (e = cudaMemcpyAsync(u_q, ka.u_q, nq * 8, kind, s->stream))) return cuda_fail(s, e, "copy u_q");
  if (u_f && (e = cudaMemcpyAsync(u_f, s->d_uf_ref, nf * 8, kind, s->stream))) return cuda_fail(s, e, "copy u_f");
  return check_flag(s);
}

// fixed-step time loop of sse_rk_steps / sse_rk_steps_snapshots: every > 0
// copies the state (and, with residuals, its residual) after every
// every-th step into the caller's buffers, in the memory kind of u
static int32_t rk_run(sse_solver *s, double *u, int32_t n_steps, double dt, int32_t scheme, double *t,
                      int32_t memory, int32_t every, double *snapshots, double *residuals) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (!u || n_steps < 0) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null u or negative n_steps");
  if (every < 0 || (every > 0 && !snapshots))
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "snapshots need every >= 1 and a snapshot buffer");
  if (scheme != SSE_CARPENTER_KENNEDY_2N54 && scheme != SSE_RK4) return fail(s, SSE_ERR_INVALID_ARGUMENT, "unknown scheme");
  const sse_config &c = s->cfg;
  size_t n = (size_t)c.n_p * c.n_c * c.n_e;
  cudaError_t e;
  double *du = u;
  if (memory == SSE_HOST) {
    if ((e = cudaMemcpyAsync(s->d_u, u, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
    du = s->d_u;
  } else if (memory != SSE_DEVICE) {
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "memory must be SSE_HOST or SSE_DEVICE");
  }
  if (scheme == SSE_RK4 && !s->d_acc) {
    void *p;
    if ((e = alloc(s, n * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_acc = (double *)p;
    if ((e = alloc(s, n * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_ust = (double *)p;
  }
  const bool mixed = s->ka.mixed;
  const bool compact = s->ka.compact != 0;
  if (compact && !s->d_ust2) {
    void *p;
    if ((e = alloc(s, n * 8, &p))) return cuda_fail(s, e, "alloc"); s->d_ust2 = (double *)p;
  }
  if (mixed && (e = cudaMemsetAsync(s->d_comp, 0, n * 8, s->stream))) return cuda_fail(s, e, "memset");
  // the mixed form picks its reference state (a synchronising reduction)
  // before any step is launched or captured
  if (mixed && n_steps > 0) {
    int rc = ensure_reference(s, du);
    if (rc != SSE_OK) return rc;
  }
  // one-kernel stages: each launch evaluates the stage's residual and
  // applies its update.  The neighbours read the stage input for their facet
  // traces, so the update goes to another buffer: CK2N54 alternates u and
  // d_ust2 (five stages end in d_ust2, copied back), RK4 alternates the
  // stage inputs d_ust and d_ust2 and writes u in place on its last stage
  auto compact_step = [&]() -> cudaError_t {
    cudaError_t err;
    CompactStage cs{};
    if (scheme == SSE_CARPENTER_KENNEDY_2N54) {
      double *buf[2] = {du, s->d_ust2};
      for (int st = 0; st < 5; ++st) {
        cs = CompactStage{};
        cs.mode = kCompactCK;
        cs.first = st == 0;
        cs.a = kCKA[st]; cs.b = kCKB[st]; cs.dt = dt;
        cs.uin = buf[st & 1];
        cs.acc = s->d_tmp;
        cs.out = buf[(st + 1) & 1];
        if ((err = launch_std_compact(s->ka, cs, s->stream))) return err;
      }
      return cudaMemcpyAsync(du, s->d_ust2, n * 8, cudaMemcpyDeviceToDevice, s->stream);
    }
    const double cst[3] = {dt / 2, dt / 2, dt};
    const double *in[4] = {du, s->d_ust, s->d_ust2, s->d_ust};
    double *out[3] = {s->d_ust, s->d_ust2, s->d_ust};
    for (int st = 0; st < 4; ++st) {
      cs = CompactStage{};
      cs.uin = in[st];
      cs.ubase = du;
      cs.acc = s->d_acc;
      if (st < 3) {
        cs.mode = kCompactRK4;
        cs.first = st == 0;
        cs.w = st == 0 ? 0.0 : 2.0;
        cs.c = cst[st];
        cs.out = out[st];
      } else {
        cs.mode = kCompactRK4Final;
        cs.c = dt / 6;
        cs.out = du;
      }
      if ((err = launch_std_compact(s->ka, cs, s->stream))) return err;
    }
    return cudaSuccess;
  };
  auto step_once = [&]() -> cudaError_t {
    cudaError_t err;
    if (compact) return compact_step();
    if (scheme == SSE_CARPENTER_KENNEDY_2N54) {
      for (int st = 0; st < 5; ++st) {
        if ((err = residual_device(s, du, s->d_dudt))) return err;
        err = mixed ? launch_ck_stage_compensated(du, s->d_comp, s->d_tmp, s->d_dudt, kCKA[st], kCKB[st],
                                                  dt, st == 0, n, s->stream)
                    : launch_ck_stage(du, s->d_tmp, s->d_dudt, kCKA[st], kCKB[st], dt, st == 0, n, s->stream);
        if (err) return err;
      }
      return cudaSuccess;
    }
    const double half = dt / 2;
    if ((err = residual_device(s, du, s->d_dudt))) return err;
    if ((err = launch_rk4_stage(du, s->d_ust, s->d_acc, s->d_dudt, 0.0, half, 1, n, s->stream))) return err;
    if ((err = residual_device(s, s->d_ust, s->d_dudt))) return err;
    if ((err = launch_rk4_stage(du, s->d_ust, s->d_acc, s->d_dudt, 2.0, half, 0, n, s->stream))) return err;
    if ((err = residual_device(s, s->d_ust, s->d_dudt))) return err;
    if ((err = launch_rk4_stage(du, s->d_ust, s->d_acc, s->d_dudt, 2.0, dt, 0, n, s->stream))) return err;
    if ((err = residual_device(s, s->d_ust, s->d_dudt))) return err;
    return launch_rk4_final(du, s->d_acc, s->d_dudt, dt / 6, n, s->stream);
  };
  // several steps: replay one captured step (one graph launch per step
  // instead of three kernel launches per stage); direct launches when the
  // stream cannot be captured (the legacy default stream)
  sse_solver::StepGraph &G = s->step_graph;
  if (n_steps >= 2) {
    const bool same = G.exec && G.u == du && G.dt == dt && G.scheme == scheme && G.mixed == (int)mixed &&
                      G.compact == (int)compact && G.stream == s->stream;
    if (!same) {
      if (G.exec) cudaGraphExecDestroy(G.exec);
      G = sse_solver::StepGraph{};
      cudaGraph_t graph = nullptr;
      if (cudaStreamBeginCapture(s->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        cudaError_t ec = step_once();
        cudaError_t ee = cudaStreamEndCapture(s->stream, &graph);
        if (ec == cudaSuccess && ee == cudaSuccess && graph &&
            cudaGraphInstantiate(&G.exec, graph, 0) == cudaSuccess) {
          G.u = du; G.dt = dt; G.scheme = scheme; G.mixed = (int)mixed; G.compact = (int)compact;
          G.stream = s->stream;
        } else {
          G.exec = nullptr;
        }
        if (graph) cudaGraphDestroy(graph);
      }
      cudaGetLastError();  // a refused capture leaves no sticky error; clear the last one
    }
  }
  const cudaMemcpyKind out_kind = memory == SSE_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  for (int step = 0; step < n_steps; ++step) {
    e = (n_steps >= 2 && G.exec) ? cudaGraphLaunch(G.exec, s->stream) : step_once();
    if (e) return cuda_fail(s, e, "step");
    if (every > 0 && (step + 1) % every == 0) {
      const size_t i = (size_t)((step + 1) / every - 1);
      if ((e = cudaMemcpyAsync(snapshots + i * n, du, n * 8, out_kind, s->stream)))
        return cuda_fail(s, e, "snapshot");
      if (residuals) {
        if ((e = residual_device(s, du, s->d_dudt))) return cuda_fail(s, e, "snapshot residual");
        if ((e = cudaMemcpyAsync(residuals + i * n, s->d_dudt, n * 8, out_kind, s->stream)))
          return cuda_fail(s, e, "snapshot residual");
      }
    }
  }
  if (memory == SSE_HOST && (e = cudaMemcpyAsync(u, s->d_u, n * 8, cudaMemcpyDeviceToHost, s->stream)))
    return cuda_fail(s, e, "D2H");
  if (t) *t += n_steps * dt;
  return check_flag(s);
}

int32_t sse_rk_steps(sse_solver *s, double *u, int32_t n_steps, double dt, int32_t scheme, double *t,
                     int32_t memory) {
  return rk_run(s, u, n_steps, dt, scheme, t, memory, 0, nullptr, nullptr);
}

int32_t sse_rk_steps_snapshots(sse_solver *s, double *u, int32_t n_steps, double dt, int32_t scheme,
                               int32_t every, double *snapshots, double *residuals, double *t,
                               int32_t memory) {
  if (every < 1) return s ? fail(s, SSE_ERR_INVALID_ARGUMENT, "every must be >= 1") : SSE_ERR_INVALID_ARGUMENT;
  return rk_run(s, u, n_steps, dt, scheme, t, memory, every, snapshots, residuals);
}

int32_t sse_residual_vjp(sse_solver *s, const double *u, const double *lam, double *mu, int32_t memory) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (!u || !lam || !mu) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null u/lam/mu");
  if (memory != SSE_HOST && memory != SSE_DEVICE)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "memory must be SSE_HOST or SSE_DEVICE");
  int rc = enable_adjoint(s);
  if (rc != SSE_OK) return rc;
  const bool mixed = s->ka.mixed != 0;
  if (mixed && (rc = enable_adjoint_mixed(s)) != SSE_OK) return rc;
  const size_t n = (size_t)s->cfg.n_p * s->cfg.n_c * s->cfg.n_e;
  cudaError_t e;
  auto run = [&](const double *du, const double *dl, double *dm) -> cudaError_t {
    return mixed ? vjp_device_mixed(s, du, dl, dm) : vjp_device(s, du, dl, dm);
  };
  if (memory == SSE_DEVICE) {
    // the mixed form picks its reference state on its first call
    if (mixed && (rc = ensure_reference(s, u)) != SSE_OK) return rc;
    if ((e = run(u, lam, mu))) return cuda_fail(s, e, "residual vjp");
  } else {
    if ((e = cudaMemcpyAsync(s->d_u, u, n * 8, cudaMemcpyHostToDevice, s->stream)) ||
        (e = cudaMemcpyAsync(s->d_lam, lam, n * 8, cudaMemcpyHostToDevice, s->stream)))
      return cuda_fail(s, e, "H2D");
    if (mixed && (rc = ensure_reference(s, s->d_u)) != SSE_OK) return rc;
    if ((e = run(s->d_u, s->d_lam, s->d_mu))) return cuda_fail(s, e, "residual vjp");
    if ((e = cudaMemcpyAsync(mu, s->d_mu, n * 8, cudaMemcpyDeviceToHost, s->stream))) return cuda_fail(s, e, "D2H");
  }
  return check_flag(s);
}

// Common set-up of a recording: validates the arguments, fixes the tape's
// scheme and precision, and returns the bytes of one checkpointed state and
// of one stage's recorded data.
static int tape_begin(sse_solver *s, double *u, int32_t n_steps, double dt, int32_t scheme, int32_t memory,
                      size_t *ckpt_state, size_t *stage_bytes) {
  if (!u || n_steps < 1) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null u or n_steps < 1");
  if (scheme != SSE_CARPENTER_KENNEDY_2N54 && scheme != SSE_RK4)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "unknown scheme");
  if (memory != SSE_HOST && memory != SSE_DEVICE)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "memory must be SSE_HOST or SSE_DEVICE");
  int rc = enable_adjoint(s);
  if (rc != SSE_OK) return rc;
  const sse_config &c = s->cfg;
  const size_t n = (size_t)c.n_p * c.n_c * c.n_e;
  const size_t nqs = (size_t)c.n_q * c.n_c * c.n_e, nfs = (size_t)c.n_f * c.n_c * c.n_e;
  sse_solver::Tape &T = s->tape;
  T.valid = false;
  T.slots_seg = -1;
  T.binomial = false;
  T.descent_intact = false;
  T.plan.clear();
  T.n_steps = n_steps;
  T.scheme = scheme;
  T.stages = scheme == SSE_RK4 ? 4 : 5;
  T.mixed = s->ka.mixed != 0;
  T.nodal = !T.mixed;
  T.dt = dt;
  *ckpt_state = (T.mixed ? 2 : 1) * n * 8;
  *stage_bytes = (n + (T.nodal ? nqs + nfs : 0)) * 8;
  return SSE_OK;
}

// Bytes of a recording with nckpt checkpointed states and the stage data of
// slot_steps steps: fixed work buffers u, tmp, comp, dudt, acc, ust, ybar,
// qbar, ybar' (every buffer padded to 256 bytes).
static size_t tape_bytes(const sse_solver *s, size_t nckpt, size_t slot_steps, size_t ckpt_state,
                         size_t stage_bytes) {
  const size_t n = (size_t)s->cfg.n_p * s->cfg.n_c * s->cfg.n_e;
  return nckpt * ckpt_state + slot_steps * s->tape.stages * stage_bytes + 9 * (n * 8 + 256) + 8 * 256;
}

// Device memory a recording may use: 3/4 of what is free (counting the
// tape's own block) less 512 MiB.
static int tape_budget(sse_solver *s, double *budget) {
  size_t free_b = 0, total_b = 0;
  cudaError_t e = cudaMemGetInfo(&free_b, &total_b);
  if (e != cudaSuccess) return cuda_fail(s, e, "cudaMemGetInfo");
  *budget = 0.75 * (double)(free_b + s->tape.capacity) - (double)((size_t)512 << 20);
  return SSE_OK;
}

// (Re)allocates the tape's block for nckpt checkpoints and slot_steps steps
// of stage data and carves it.
static int tape_alloc(sse_solver *s, size_t nckpt, size_t slot_steps, size_t ckpt_state, size_t stage_bytes,
                      const char *hint) {
  sse_solver::Tape &T = s->tape;
  const sse_config &c = s->cfg;
  const size_t n = (size_t)c.n_p * c.n_c * c.n_e;
  const size_t nqs = (size_t)c.n_q * c.n_c * c.n_e, nfs = (size_t)c.n_f * c.n_c * c.n_e;
  const size_t bytes = tape_bytes(s, nckpt, slot_steps, ckpt_state, stage_bytes);
  cudaError_t e;
  if (bytes > T.capacity) {
    // grow: release the old block first, then check what is free
    if (s->stream && (e = cudaStreamSynchronize(s->stream))) return cuda_fail(s, e, "sync");
    if (T.block) cudaFree(T.block);
    T.block = nullptr;
    T.capacity = 0;
    size_t free_b = 0, total_b = 0;
    if ((e = cudaMemGetInfo(&free_b, &total_b))) return cuda_fail(s, e, "cudaMemGetInfo");
    if (bytes + ((size_t)256 << 20) > free_b)
      return fail(s, SSE_ERR_OUT_OF_MEMORY,
                  "recording needs " + std::to_string(bytes >> 20) + " MiB of device memory, " +
                      std::to_string(free_b >> 20) + " MiB free (" + hint + ")");
    if ((e = cudaMalloc(&T.block, bytes))) {
      T.block = nullptr;
      return fail(s, SSE_ERR_OUT_OF_MEMORY, std::string("recording: ") + cudaGetErrorString(e));
    }
    T.capacity = bytes;
  }
  T.bytes = bytes;
  char *cur = (char *)T.block;
  auto carve = [&](size_t count) {
    double *p = (double *)cur;
    cur += (count * 8 + 255) / 256 * 256;
    return p;
  };
  const size_t slots = slot_steps * T.stages;
  T.ckpt = carve(nckpt * n);
  T.ckpt_comp = T.mixed ? carve(nckpt * n) : nullptr;
  T.seg_y = carve(slots * n);
  T.seg_uq = T.nodal ? carve(slots * nqs) : nullptr;
  T.seg_uf = T.nodal ? carve(slots * nfs) : nullptr;
  T.w_u = carve(n); T.w_tmp = carve(n); T.w_comp = carve(n); T.w_dudt = carve(n);
  T.w_acc = carve(n); T.w_ust = carve(n); T.ybar = carve(n); T.qbar = carve(n); T.yp = carve(n);
  return SSE_OK;
}

// Copies between the working state (and the mixed form's compensation) and
// checkpoint slot g.
static cudaError_t tape_save(sse_solver *s, const double *u, size_t g) {
  sse_solver::Tape &T = s->tape;
  const size_t n = (size_t)s->cfg.n_p * s->cfg.n_c * s->cfg.n_e;
  cudaError_t e = cudaMemcpyAsync(T.ckpt + g * n, u, n * 8, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess && T.mixed)
    e = cudaMemcpyAsync(T.ckpt_comp + g * n, T.w_comp, n * 8, cudaMemcpyDeviceToDevice, s->stream);
  return e;
}

static cudaError_t tape_load(sse_solver *s, size_t g) {
  sse_solver::Tape &T = s->tape;
  const size_t n = (size_t)s->cfg.n_p * s->cfg.n_c * s->cfg.n_e;
  cudaError_t e = cudaMemcpyAsync(T.w_u, T.ckpt + g * n, n * 8, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess && T.mixed)
    e = cudaMemcpyAsync(T.w_comp, T.ckpt_comp + g * n, n * 8, cudaMemcpyDeviceToDevice, s->stream);
  return e;
}

// Reverse of one recorded step whose stage data sits in slots q0 ..
// q0 + stages - 1: ybar <- (du_{i+1}/du_i)^T ybar.
static cudaError_t reverse_step(sse_solver *s, size_t q0) {
  sse_solver::Tape &T = s->tape;
  const sse_config &c = s->cfg;
  const size_t n = (size_t)c.n_p * c.n_c * c.n_e;
  const size_t nqs = (size_t)c.n_q * c.n_c * c.n_e, nfs = (size_t)c.n_f * c.n_c * c.n_e;
  const double dt = T.dt;
  auto stage_vjp = [&](size_t q, const double *lam) -> cudaError_t {
    if (T.mixed) return vjp_device_mixed(s, T.seg_y + q * n, lam, s->d_mu);
    const double *uq = T.nodal ? T.seg_uq + q * nqs : nullptr;
    const double *uf = T.nodal ? T.seg_uf + q * nfs : nullptr;
    return vjp_device(s, T.seg_y + q * n, lam, s->d_mu, uq, uf);
  };
  cudaError_t e;
  if (T.scheme == SSE_CARPENTER_KENNEDY_2N54) {
    e = launch_adj_lincomb(T.qbar, T.ybar, 0.0, kCKB[4], n, s->stream);
    for (int st = 4; st >= 0 && e == cudaSuccess; --st) {
      e = stage_vjp(q0 + st, T.qbar);
      if (e == cudaSuccess)
        e = launch_adj_ck_stage(T.ybar, T.qbar, s->d_mu, dt, kCKA[st], st > 0 ? kCKB[st - 1] : 0.0, n, s->stream);
    }
    return e;
  }
  // u' = u + dt/6 (k1 + 2 k2 + 2 k3 + k4), stages y1 = u, y2 = u + dt/2 k1,
  // y3 = u + dt/2 k2, y4 = u + dt k3
  e = cudaMemcpyAsync(T.yp, T.ybar, n * 8, cudaMemcpyDeviceToDevice, s->stream);
  if (e == cudaSuccess) e = launch_adj_lincomb(T.qbar, T.ybar, 0.0, dt / 6, n, s->stream);
  const double cy[4] = {0.0, dt / 6, dt / 3, dt / 3};  // kbar of stage st-1: cy ybar' + cm mu
  const double cm[4] = {0.0, dt / 2, dt / 2, dt};
  for (int st = 3; st >= 0 && e == cudaSuccess; --st) {
    e = stage_vjp(q0 + st, T.qbar);
    if (e == cudaSuccess)
      e = launch_adj_rk4_stage(T.ybar, T.qbar, s->d_mu, T.yp, cy[st], cm[st], st == 0, n, s->stream);
  }
  return e;
}

int32_t sse_rk_record(sse_solver *s, double *u, int32_t n_steps, double dt, int32_t scheme,
                      int32_t checkpoint_every, double *t, int32_t memory) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (checkpoint_every < 0) return fail(s, SSE_ERR_INVALID_ARGUMENT, "negative checkpoint_every");
  size_t ckpt_state = 0, stage_bytes = 0;
  int rc = tape_begin(s, u, n_steps, dt, scheme, memory, &ckpt_state, &stage_bytes);
  if (rc != SSE_OK) return rc;
  const size_t n = (size_t)s->cfg.n_p * s->cfg.n_c * s->cfg.n_e;
  sse_solver::Tape &T = s->tape;
  auto need = [&](int every) {
    const size_t nseg = (n_steps + every - 1) / every;
    return tape_bytes(s, nseg, every, ckpt_state, stage_bytes);
  };
  cudaError_t e;
  int every = checkpoint_every > 0 ? std::min(checkpoint_every, (int)n_steps) : 1;
  if (checkpoint_every == 0) {
    // the longest segments that fit: fewest segments to recompute in the
    // reverse sweep
    double budget = 0;
    if ((rc = tape_budget(s, &budget)) != SSE_OK) return rc;
    for (int c2 = n_steps; c2 >= 1; --c2)
      if ((double)need(c2) <= budget) { every = c2; break; }
  }
  T.every = every;
  T.nseg = (n_steps + every - 1) / every;
  if ((rc = tape_alloc(s, T.nseg, every, ckpt_state, stage_bytes, "choose another checkpoint_every")) != SSE_OK)
    return rc;
  double *du = u;
  if (memory == SSE_HOST) {
    if ((e = cudaMemcpyAsync(s->d_u, u, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
    du = s->d_u;
  }
  if (T.mixed && (e = cudaMemsetAsync(T.w_comp, 0, n * 8, s->stream))) return cuda_fail(s, e, "memset");
  for (int step = 0; step < n_steps; ++step) {
    if (step % every == 0 && (e = tape_save(s, du, step / every))) return cuda_fail(s, e, "checkpoint");
    // the last segment's stage data is kept from this run: the reverse
    // sweep starts without recomputing it
    const int last0 = (T.nseg - 1) * every;
    if ((e = tape_step(s, du, step >= last0 ? step - last0 : -1))) return cuda_fail(s, e, "step");
  }
  if (memory == SSE_HOST && (e = cudaMemcpyAsync(u, s->d_u, n * 8, cudaMemcpyDeviceToHost, s->stream)))
    return cuda_fail(s, e, "D2H");
  if (t) *t += n_steps * dt;
  rc = check_flag(s);
  T.valid = rc == SSE_OK;
  T.slots_seg = T.nseg - 1;
  return rc;
}

int32_t sse_rk_record_binomial(sse_solver *s, double *u, int32_t n_steps, double dt, int32_t scheme,
                               int32_t n_checkpoints, double *t, int32_t memory) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (n_checkpoints < 0) return fail(s, SSE_ERR_INVALID_ARGUMENT, "negative n_checkpoints");
  size_t ckpt_state = 0, stage_bytes = 0;
  int rc = tape_begin(s, u, n_steps, dt, scheme, memory, &ckpt_state, &stage_bytes);
  if (rc != SSE_OK) return rc;
  const size_t n = (size_t)s->cfg.n_p * s->cfg.n_c * s->cfg.n_e;
  sse_solver::Tape &T = s->tape;
  int c = std::min(n_checkpoints, n_steps - 1);
  if (n_checkpoints == 0) {
    // as many checkpoints as the budget holds (at most one per step)
    double budget = 0;
    if ((rc = tape_budget(s, &budget)) != SSE_OK) return rc;
    c = 0;
    for (int k = n_steps - 1; k >= 0; --k)
      if ((double)tape_bytes(s, (size_t)k + 1, 1, ckpt_state, stage_bytes) <= budget) { c = k; break; }
  }
  if ((rc = tape_alloc(s, (size_t)c + 1, 1, ckpt_state, stage_bytes, "choose fewer checkpoints")) != SSE_OK)
    return rc;
  T.binomial = true;
  T.ckpts = c;
  T.every = 0;
  T.nseg = c + 1;
  {
    BinomialTable tab;
    tab.build(n_steps, c);
    T.plan.clear();
    T.plan_steps = binomial_plan(0, n_steps, c, 0, tab, T.plan);
  }
  cudaError_t e;
  double *du = u;
  if (memory == SSE_HOST) {
    if ((e = cudaMemcpyAsync(s->d_u, u, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
    du = s->d_u;
  }
  if (T.mixed && (e = cudaMemsetAsync(T.w_comp, 0, n * 8, s->stream))) return cuda_fail(s, e, "memset");
  if ((e = tape_save(s, du, 0))) return cuda_fail(s, e, "checkpoint");
  // the first descent of the schedule: advance and keep checkpoints down to
  // the last step, which is taken with its stage data recorded
  size_t i = 0;
  for (; i < T.plan.size() && e == cudaSuccess; ++i) {
    const int a = T.plan[i], k = act_kind(a), arg = act_arg(a);
    if (k == kActLoad) e = tape_load(s, arg);
    else if (k == kActStore) e = tape_save(s, T.w_u, arg);
    else if (k == kActAdvance) for (int j = 0; j < arg && e == cudaSuccess; ++j) e = tape_step(s, T.w_u, -1);
    else { e = tape_step(s, T.w_u, 0); break; }
  }
  if (e != cudaSuccess) return cuda_fail(s, e, "recording");
  T.plan_pos = i;
  if ((e = cudaMemcpyAsync(du, T.w_u, n * 8, cudaMemcpyDeviceToDevice, s->stream))) return cuda_fail(s, e, "state");
  if (memory == SSE_HOST && (e = cudaMemcpyAsync(u, s->d_u, n * 8, cudaMemcpyDeviceToHost, s->stream)))
    return cuda_fail(s, e, "D2H");
  if (t) *t += n_steps * dt;
  rc = check_flag(s);
  T.valid = rc == SSE_OK;
  T.descent_intact = T.valid;
  return rc;
}

int32_t sse_rk_adjoint(sse_solver *s, const double *lam_T, double *lam_0, double *out_info, int32_t memory) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (!lam_T || !lam_0) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null lam_T/lam_0");
  if (memory != SSE_HOST && memory != SSE_DEVICE)
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "memory must be SSE_HOST or SSE_DEVICE");
  sse_solver::Tape &T = s->tape;
  if (!T.valid) return fail(s, SSE_ERR_INVALID_ARGUMENT, "no recorded trajectory (call sse_rk_record first)");
  const sse_config &c = s->cfg;
  const size_t n = (size_t)c.n_p * c.n_c * c.n_e;
  cudaError_t e;
  cudaMemcpyKind kin = memory == SSE_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
  if ((e = cudaMemcpyAsync(T.ybar, lam_T, n * 8, kin, s->stream))) return cuda_fail(s, e, "copy lam_T");
  // the recomputation runs in the recorded precision; the stage adjoints in FP64
  const int saved_mixed = s->ka.mixed;
  s->ka.mixed = T.mixed ? 1 : 0;
  if (T.mixed) {
    int rc = enable_adjoint_mixed(s);
    if (rc != SSE_OK) { s->ka.mixed = saved_mixed; return rc; }
  }
  long long recomputed = 0;
  if (T.binomial) {
    // the schedule's actions; the leaf the recording run took is reversed
    // from its stage data while the descent's checkpoints are intact
    size_t i = 0;
    if (T.descent_intact) {
      e = reverse_step(s, 0);
      i = T.plan_pos + 1;
    }
    for (; i < T.plan.size() && e == cudaSuccess; ++i) {
      const int a = T.plan[i], k = act_kind(a), arg = act_arg(a);
      if (k == kActLoad) {
        e = tape_load(s, arg);
      } else if (k == kActStore) {
        e = tape_save(s, T.w_u, arg);
      } else if (k == kActAdvance) {
        for (int j = 0; j < arg && e == cudaSuccess; ++j) e = tape_step(s, T.w_u, -1);
        recomputed += arg;
      } else {
        e = tape_step(s, T.w_u, 0);
        if (e == cudaSuccess) e = reverse_step(s, 0);
        ++recomputed;
      }
    }
    T.descent_intact = false;  // the reversal reused the descent's slots
  } else {
    for (int seg = T.nseg - 1; seg >= 0 && e == cudaSuccess; --seg) {
      const int s0 = seg * T.every, m = std::min(T.n_steps, s0 + T.every) - s0;
      if (T.slots_seg != seg) {
        // recompute the segment from its checkpoint, storing its stage data
        T.slots_seg = -1;
        e = tape_load(s, seg);
        for (int i = 0; i < m && e == cudaSuccess; ++i) e = tape_step(s, T.w_u, i);
        if (e == cudaSuccess) T.slots_seg = seg;
        ++recomputed;
      }
      for (int i = m - 1; i >= 0 && e == cudaSuccess; --i) e = reverse_step(s, (size_t)i * T.stages);
    }
  }
  s->ka.mixed = saved_mixed;
  if (e != cudaSuccess) return cuda_fail(s, e, "adjoint sweep");
  cudaMemcpyKind kout = memory == SSE_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice;
  if ((e = cudaMemcpyAsync(lam_0, T.ybar, n * 8, kout, s->stream))) return cuda_fail(s, e, "copy lam_0");
  if (out_info) {
    out_info[0] = T.nseg;
    out_info[1] = T.binomial ? -1 : T.every;
    out_info[2] = (double)T.bytes;
    out_info[3] = (double)recomputed;
  }
  return check_flag(s);
}

// Forward steps (beyond the recorded ones) of the optimal binomial schedule
// for n_steps steps and n_checkpoints free slots; host only.
int32_t sse_binomial_schedule(int32_t n_steps, int32_t n_checkpoints, int64_t *extra_steps,
                              int32_t *first_split) {
  if (n_steps < 1 || n_checkpoints < 0 || !extra_steps) return SSE_ERR_INVALID_ARGUMENT;
  const int c = std::min(n_checkpoints, n_steps - 1);
  BinomialTable tab;
  tab.build(n_steps, c);
  std::vector<int> plan;
  const long long steps = binomial_plan(0, n_steps, c, 0, tab, plan);
  *extra_steps = steps - n_steps;
  if (first_split) *first_split = n_steps > 1 && c > 0 ? tab.split(n_steps, c) : 0;
  return SSE_OK;
}

int32_t sse_conservation_residual(sse_solver *s, const double *u, const double *dudt, double *out,
                                  int32_t memory) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (!u || !dudt || !out) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null argument");
  const sse_config &c = s->cfg;
  size_t n = (size_t)c.n_p * c.n_c * c.n_e;
  cudaError_t e;
  const double *du = u, *dd = dudt;
  if (memory == SSE_HOST) {
    if ((e = cudaMemcpyAsync(s->d_u, u, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
    if ((e = cudaMemcpyAsync(s->d_tmp, dudt, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
    du = s->d_u;
    dd = s->d_tmp;
  } else if (memory != SSE_DEVICE) {
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "memory must be SSE_HOST or SSE_DEVICE");
  }
  if ((e = launch_conservation(s->ka, du, dd, s->d_partial, s->stream))) return cuda_fail(s, e, "conservation");
  std::vector<double> part((size_t)c.n_e * (c.n_c + 1));
  if ((e = cudaMemcpyAsync(part.data(), s->d_partial, part.size() * 8, cudaMemcpyDeviceToHost, s->stream)))
    return cuda_fail(s, e, "D2H");
  if ((e = cudaStreamSynchronize(s->stream))) return cuda_fail(s, e, "sync");
  for (int q = 0; q <= c.n_c; ++q) out[q] = 0.0;
  for (int k = 0; k < c.n_e; ++k)
    for (int q = 0; q <= c.n_c; ++q) out[q] += part[(size_t)k * (c.n_c + 1) + q];
  return SSE_OK;
}

int32_t sse_energy_residual(sse_solver *s, const double *u, const double *dudt, double *out,
                            int32_t memory) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (!u || !dudt || !out) return fail(s, SSE_ERR_INVALID_ARGUMENT, "null argument");
  const sse_config &c = s->cfg;
  if ((size_t)s->ka.epb * s->ka.layE.team_doubles * sizeof(double) > 220 * 1024)
    return fail(s, SSE_ERR_UNSUPPORTED, "element too large for the energy analysis");
  size_t n = (size_t)c.n_p * c.n_c * c.n_e;
  cudaError_t e;
  const double *du = u, *dd = dudt;
  if (memory == SSE_HOST) {
    if ((e = cudaMemcpyAsync(s->d_u, u, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
    if ((e = cudaMemcpyAsync(s->d_tmp, dudt, n * 8, cudaMemcpyHostToDevice, s->stream))) return cuda_fail(s, e, "H2D");
    du = s->d_u;
    dd = s->d_tmp;
  } else if (memory != SSE_DEVICE) {
    return fail(s, SSE_ERR_INVALID_ARGUMENT, "memory must be SSE_HOST or SSE_DEVICE");
  }
  if ((e = cudaMemsetAsync(s->d_flag, 0, sizeof(int), s->stream))) return cuda_fail(s, e, "memset");
  if ((e = launch_energy(s->ka, du, dd, s->d_partial, s->stream))) return cuda_fail(s, e, "energy");
  std::vector<double> part((size_t)c.n_e * c.n_c);
  int flag = 0;
  if ((e = cudaMemcpyAsync(part.data(), s->d_partial, part.size() * 8, cudaMemcpyDeviceToHost, s->stream)) ||
      (e = cudaMemcpyAsync(&flag, s->d_flag, sizeof(int), cudaMemcpyDeviceToHost, s->stream)))
    return cuda_fail(s, e, "D2H");
  if ((e = cudaStreamSynchronize(s->stream))) return cuda_fail(s, e, "sync");
  if (flag) return fail(s, SSE_ERR_NONPHYSICAL, "an element mass matrix is not positive definite");
  for (int q = 0; q < c.n_c; ++q) out[q] = 0.0;
  for (int k = 0; k < c.n_e; ++k)
    for (int q = 0; q < c.n_c; ++q) out[q] += part[(size_t)k * c.n_c + q];
  return SSE_OK;
}

// Average device time (ms) of each residual phase over n_iter evaluations,
// timed with CUDA events on the handle's stream: out[0] = phase A (nodal
// values), out[1] = phase B (time derivative), out[2] = one RK stage update.
int32_t sse_phase_timings(sse_solver *s, const double *u_dev, int32_t n_iter, double *out) {
  if (!s || !u_dev || !out || n_iter <= 0) return SSE_ERR_INVALID_ARGUMENT;
  if (s->ka.mixed) {
    int rc = ensure_reference(s, u_dev);
    if (rc != SSE_OK) return rc;
  }
  KernelArgs ka = s->ka;
  ka.u = u_dev;
  ka.dudt = s->d_dudt;
  size_t n = (size_t)s->cfg.n_p * s->cfg.n_c * s->cfg.n_e;
  cudaEvent_t ev[4];
  for (int i = 0; i < 4; ++i) cudaEventCreate(&ev[i]);
  float ta = 0, tb = 0, tc = 0;
  cudaError_t e = cudaSuccess;
  CompactStage cst{};
  cst.mode = kCompactResidual;
  cst.uin = u_dev;
  cst.out = s->d_dudt;
  for (int it = 0; it < n_iter && e == cudaSuccess; ++it) {
    cudaEventRecord(ev[0], s->stream);
    // the one-kernel StandardForm path has no separate phase A (out[0] = 0)
    if (!ka.compact) e = launch_nodal_values(ka, s->stream);
    cudaEventRecord(ev[1], s->stream);
    if (e == cudaSuccess) e = ka.compact ? launch_std_compact(ka, cst, s->stream) : launch_time_derivative(ka, s->stream);
    cudaEventRecord(ev[2], s->stream);
    // stage update into the host-staging buffer (never the caller's state)
    if (e == cudaSuccess && s->d_u != u_dev)
      e = launch_ck_stage(s->d_u, s->d_tmp, s->d_dudt, 0.5, 0.0, 1e-300, 0, n, s->stream);
    cudaEventRecord(ev[3], s->stream);
    if (e == cudaSuccess) e = cudaEventSynchronize(ev[3]);
    float a, b, c2;
    cudaEventElapsedTime(&a, ev[0], ev[1]);
    cudaEventElapsedTime(&b, ev[1], ev[2]);
    cudaEventElapsedTime(&c2, ev[2], ev[3]);
    ta += a; tb += b; tc += c2;
  }
  for (int i = 0; i < 4; ++i) cudaEventDestroy(ev[i]);
  if (e != cudaSuccess) return cuda_fail(s, e, "timing");
  out[0] = ka.compact ? 0.0 : ta / n_iter;
  out[1] = tb / n_iter;
  out[2] = tc / n_iter;
  return check_flag(s);
}

int32_t sse_kernel_path(const sse_solver *s) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  return s->ka.compact ? SSE_PATH_ONE_KERNEL : SSE_PATH_TWO_PHASE;
}

int32_t sse_set_kernel_path(sse_solver *s, int32_t path) {
  if (!s) return SSE_ERR_INVALID_ARGUMENT;
  if (path == SSE_PATH_TWO_PHASE) {
    s->ka.compact = 0;
    return SSE_OK;
  }
  if (path != SSE_PATH_ONE_KERNEL) return fail(s, SSE_ERR_INVALID_ARGUMENT, "unknown kernel path");
  if (!s->compact_ok)
    return fail(s, SSE_ERR_UNSUPPORTED,
                "the one-kernel path covers StandardForm with at most 32 volume, facet and modal nodes per element");
  s->ka.compact = 1;
  return SSE_OK;
}

// sizeof checks for foreign-language bindings
int32_t sse_struct_sizes(int32_t *out) {
  out[0] = (int32_t)sizeof(sse_config);
  out[1] = (int32_t)sizeof(sse_csc);
  out[2] = (int32_t)sizeof(sse_operators);
  out[3] = (int32_t)sizeof(sse_geometry);
  out[4] = (int32_t)sizeof(sse_metric_operators);
  out[5] = (int32_t)sizeof(sse_geometric_factors_out);
  return 6;
}

int32_t sse_project_function(int32_t n_p, int32_t n_q, int32_t n_c, int64_t n_e,
                             const double *VDM, const double *W, const double *J_q,
                             const double *u_q, double *u0, int32_t memory) {
  g_create_error.clear();
  try {
    return project_function_run(n_p, n_q, n_c, n_e, VDM, W, J_q, u_q, u0, memory, &g_create_error);
  } catch (const std::exception &ex) {
    g_create_error = ex.what();
    return SSE_ERR_OUT_OF_MEMORY;
  }
}

int32_t sse_geometric_factors(const sse_metric_operators *ops, int64_t n_e,
                              const double *const *xyz,
                              const sse_geometric_factors_out *out, int32_t memory) {
  g_create_error.clear();
  try {
    return geometric_factors_run(ops, n_e, xyz, out, memory, &g_create_error);
  } catch (const std::exception &ex) {
    g_create_error = ex.what();
    return SSE_ERR_OUT_OF_MEMORY;
  }
}

}  // extern "C"
