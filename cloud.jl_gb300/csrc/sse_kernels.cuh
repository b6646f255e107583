// sse_kernels.cuh -- kernel argument block and launchers.
#pragma once

#include <cstddef>
#include <string>
#include <cuda_runtime.h>

#include "../../include/sse_gb300.h"
#include "sse_device.cuh"

namespace sse {

// Nodes (volume plus facet) a thread of an element team handles in the
// chunked pair passes: n_q + n_f <= kMaxNodeSlots * threads per element.
constexpr int kMaxNodeSlots = 4;

// Per-team shared-memory layout (offsets in doubles) computed on the host.
struct Layout {
  int off[12];
  int team_doubles;
};

struct KernelArgs {
  DevOps op;
  DevGeo geo;
  Physics ph;
  Layout layA, layB;
  Layout layBm;      // mixed-form phase B layout, offsets and team size in floats:
                     // 0 volume states (then r_q), 1 facet states, 2 facet fluxes,
                     // 3 mass operator, 4 pair buffer, 5 Lambda_q, 6 halfnJq,
                     // 7 primitives, 8 facet geometry, 9 reference residual,
                     // 10 mbarrier; a zero-sized optional region is read from
                     // global memory instead
  Layout layAm;      // mixed-form phase A layout (doubles; FP32 arrays from off[4], in floats)
  Layout layP1;      // projection of the constant function (NC = 1), doubles
  int ne, epb, tpb;
  const double *Ak;  // per-element weight-adjusted mass operators (n_p x n_p, column-major), or null
  const float *Akf;  // their FP32 roundings for the mixed form (row-major), or null
  // mixed form: per-element tail operators E_k = A_k V^T [I | -R^T] (n_p rows,
  // the volume then facet nodes as columns, padded to ek_quads column quads;
  // float4 (q, r) = E_k[r, 4q .. 4q+3]), or null
  const float *Ekf;
  int ek_quads;
  int fd, project_entropy, mass_wa;
  const double *u;   // modal state (np x nc x ne)
  double *dudt;      // residual   (np x nc x ne)
  double *u_q;       // volume nodal scratch (nq x nc x ne)
  double *u_f;       // facet nodal scratch, internal layout (nf x nc x ne) element-major
  float *u_qf;       // mixed form: FP32 perturbations of u_q from the reference state
  float *u_ff;       // mixed form: FP32 perturbations of u_f
  int mixed;         // 1: phase A writes u_qf/u_ff and phase B runs in FP32
  int *flag;         // nonzero: non-physical state met
  // discrete adjoint (vector-Jacobian product of the FP64 residual)
  const double *lam; // cotangent of dudt            (np x nc x ne)
  double *mu;        // result (dR/du)^T lam          (np x nc x ne)
  double *rbar_q;    // adjoint of r_q                (nq x nc x ne)
  double *gbar_f;    // adjoint of the interface flux  (nf x nc x ne, element-major)
  double *ubar_q;    // adjoint of u_q                (nq x nc x ne)
  double *ubar_f;    // adjoint of u_f                (nf x nc x ne, element-major)
  Layout layAdjB1, layAdjB2, layAdjA;
  Layout layAdjS;                          // StandardForm flux-transpose layout
  Layout layE;                             // energy_kernel layout (doubles)
  Layout layAdjG;                          // conservative-two-point pair-transpose layout
  int pair_chunk;    // pairs per shared-memory chunk in the pair-adjoint passes
  int pair_chunk_generic;  // the same for the conservative two-point flux
  int fd_chunk;      // pairs per chunk in the FP64 flux-differencing passes
  int vp_split;      // volume pairs per interface lane in the one-chunk pass (0: even split)
  int epb_bm;        // elements per block of the FP32 phase-B kernel (blocks of tpb threads)
  int epb_am;        // elements per block of the mixed phase-A kernel (blocks of tpb threads)
  int epb_a;         // elements per block of the FP64 phase-A kernel (blocks of tpb threads)
  int vdm_zsz;       // doubles of the first sum-factorisation scratch (even)
  int fd_chunk_mixed;  // pairs per chunk in the mixed-form FP32 passes
  Layout layAdjB1m, layAdjB2m, layAdjAm;  // mixed-form VJP layouts (floats)
  int pair_chunk_mixed;  // pairs per chunk in the mixed-form pair-adjoint passes
  int vdm_zsz_mixed;   // floats of the first sum-factorisation scratch (multiple of 4)
  // one-kernel StandardForm path (std_compact_kernel) for elements with at
  // most 32 volume, facet and modal nodes: one warp per element, the dense
  // operators staged once per block in shared memory
  int compact;         // 1: residuals and stages run std_compact_kernel
  const double *cops;  // packed dense operators (column-major, leading dimension = rows)
  int cop_off[12];     // offsets (doubles): kCopV, kCopVR, kCopVT, kCopR, kCopRT, kCopD + m, kCopDT + m
  int cop_doubles;     // total doubles of the packed operators (even)
  int cop_w[12];       // 0: dense (column-major); > 0: padded-row (ELL) width of a sparse operator
  int cop_i[12];       // ELL operators: offset of their column indices in copi
  const int *copi;     // ELL column indices (same layout as the values)
  int copi_ints;       // total ints of copi (a multiple of 4)
  int ct_off[10];      // per-element shared-memory offsets (doubles), kCt* below
  int ct_doubles;      // doubles per element (even)
  int epb_c;           // elements (warps) per block of std_compact_kernel

  __device__ __forceinline__ void flag_nonphysical() const { atomicOr(flag, 1); }
  // a bounded wait on a device copy gave up (reported as SSE_ERR_CUDA)
  __device__ __forceinline__ void flag_timeout() const { atomicOr(flag, 2); }
};

// most elements (warps) per block of std_compact_kernel
constexpr int kMaxCompactEpb = 8;
// packed dense operators of the compact StandardForm path
enum { kCopV = 0, kCopVR = 1, kCopVT = 2, kCopR = 3, kCopRT = 4, kCopD = 5, kCopDT = 8 };
// per-element shared-memory regions of std_compact_kernel: modal state
// followed by the neighbours' modal states (one per face; kCtUN unused),
// volume states, physical fluxes f_n, contracted fluxes g_m, facet fluxes,
// volume residual, modal residual, and the bulk-copied halfWLambda and mass
// operator (each with 32 spare bytes for its 16-byte-aligned span)
enum { kCtU = 0, kCtUN, kCtUQ, kCtF, kCtG, kCtFF, kCtRQ, kCtBM, kCtHW, kCtAK };

// what std_compact_kernel writes after the element's residual k:
//   kCompactResidual  out = k
//   kCompactRK4       acc = first ? k : acc + w k ;  out = ubase + c k
//   kCompactRK4Final  out = ubase + c (acc + k)           (out may be ubase)
//   kCompactCK        t = first ? dt k : a acc + dt k ; acc = t ; out = uin + b t
// out never aliases uin, which the neighbours read for their facet traces.
enum { kCompactResidual = 0, kCompactRK4 = 1, kCompactRK4Final = 2, kCompactCK = 3 };
struct CompactStage {
  int mode, first;
  double a, b, c, w, dt;
  const double *uin;    // the stage's input state (this element and its neighbours)
  const double *ubase;  // RK4: the step's initial state
  double *acc;          // RK4 accumulator / CK2N54 register
  double *out;
};

cudaError_t sse_set_smem_limits(const KernelArgs &ka, size_t smA, size_t smB);
cudaError_t sse_set_smem_limit_compact(const KernelArgs &ka, size_t bytes);
cudaError_t launch_std_compact(const KernelArgs &ka, const CompactStage &st, cudaStream_t s);
// column a of V (np blocks; V applied to the unit vectors), nq x np column-major
cudaError_t launch_dense_vdm(const KernelArgs &ka, double *out, cudaStream_t s);
cudaError_t sse_set_smem_limit_mixed(const KernelArgs &ka, size_t smBm);
// resident blocks per SM of the mixed phase-B kernel with smBm bytes of
// dynamic shared memory (registers, threads and shared memory together)
cudaError_t sse_mixed_b_blocks_per_sm(const KernelArgs &ka, size_t smBm, int *blocks);
cudaError_t launch_ck_stage_compensated(double *u, double *comp, double *tmp, const double *k,
                                        double a, double b, double dt, int first, size_t n,
                                        cudaStream_t st);
// out = (float)(in + shift)
cudaError_t launch_round_to_float(const double *in, float *out, size_t n, cudaStream_t st, double shift = 0.0);
// FP64 Lambda_q (n_q x d x d per element) rounded to FP32, node-major with
// lambda_stride(d) floats per node
cudaError_t launch_lambda_node_major(const double *in, float *out, size_t ne, int nq, int d, cudaStream_t st);
// the mixed phase B's packed pair tables: 4 floats per volume pair, 2 per
// facet pair
cudaError_t launch_pack_pairs(const DevOps &op, float *vpk, float *fpk, cudaStream_t st);
// FP64 halfnJq (d x nfac x n_q per element) rounded to FP32 and transposed to
// (f d + m) n_q + i
cudaError_t launch_halfnjq_transpose(const double *in, float *out, size_t ne, int nq, int d, int nfac,
                                     cudaStream_t st);
cudaError_t launch_fill_constant_state(double *buf, int nodes, int nc, size_t ne, const double *state,
                                       cudaStream_t st);
cudaError_t launch_round_transpose(const double *in, float *out, size_t nmat, int n, cudaStream_t st);
// the mixed form's per-element tail operators (KernelArgs::Ekf) from the
// FP64 mass operators ka.Ak and the dense V (Vd, n_q x n_p column-major);
// M is FP64 scratch of n_p x 4 quads doubles
cudaError_t launch_tail_operators(const KernelArgs &ka, const double *Vd, double *M, float *E, int quads,
                                  cudaStream_t st);
cudaError_t launch_nodal_values(const KernelArgs &ka, cudaStream_t st);
cudaError_t launch_projection_of_one(const KernelArgs &ka, double *P1, double *RP1, cudaStream_t st);
cudaError_t sse_set_smem_limits_mixed_a(const KernelArgs &ka);
cudaError_t launch_time_derivative(const KernelArgs &ka, cudaStream_t st);
cudaError_t launch_mass_operator(const KernelArgs &ka, double *Ak, cudaStream_t st);
cudaError_t launch_energy(const KernelArgs &ka, const double *u, const double *dudt, double *partial,
                          cudaStream_t st);
cudaError_t launch_conservation(const KernelArgs &ka, const double *u, const double *dudt,
                                double *partial, cudaStream_t st);
cudaError_t launch_ck_stage(double *u, double *tmp, const double *k, double a, double b, double dt,
                            int first, size_t n, cudaStream_t st);
cudaError_t launch_rk4_stage(const double *u, double *ust, double *acc, const double *k,
                             double acc_w, double c, int first, size_t n, cudaStream_t st);
cudaError_t launch_rk4_final(double *u, const double *acc, const double *k, double dt6, size_t n,
                             cudaStream_t st);
cudaError_t launch_facet_layout(const double *in, double *out, int nf, int ne, int nc,
                                cudaStream_t st);

// discrete adjoint (sse_adjoint.cu)
cudaError_t sse_set_smem_limits_adjoint(const KernelArgs &ka);
cudaError_t launch_residual_vjp_kernels(const KernelArgs &ka, cudaStream_t st);
cudaError_t sse_set_smem_limits_adjoint_mixed(const KernelArgs &ka);
cudaError_t launch_residual_vjp_mixed_kernels(const KernelArgs &ka, cudaStream_t st);
cudaError_t launch_adj_ck_stage(double *ybar, double *qbar, const double *mu, double dt, double a,
                                double b_prev, size_t n, cudaStream_t st);
cudaError_t launch_adj_lincomb(double *y, const double *x, double alpha, double beta, size_t n,
                               cudaStream_t st);
cudaError_t launch_adj_rk4_stage(double *ybar, double *kbar, const double *mu, const double *yp,
                                 double cy, double cm, int last, size_t n, cudaStream_t st);

// GeometricFactors on the device (sse_geometry.cu); returns an sse_status
// and leaves a message in *err on failure.
int geometric_factors_run(const sse_metric_operators *ops, int64_t n_e, const double *const *xyz,
                          const sse_geometric_factors_out *out, int memory, std::string *err);

// project_function on the device (sse_project.cu); returns an sse_status.
int project_function_run(int np, int nq, int nc, int64_t ne, const double *V, const double *W,
                         const double *J, const double *uq, double *u0, int memory, std::string *err);

}  // namespace sse
