// sse_compact.cu -- one-kernel StandardForm residual (and Runge-Kutta stage)
// for elements with at most 32 volume, facet and modal nodes.
//
// time_derivative! for StandardForm (standard_form_first_order.jl:16-63)
// together with the nodal_values! that precedes it
// (standard_form_first_order.jl:1-14): the facet traces u_f = R V u are
// evaluated inside the kernel, for the element and, from their modal
// coefficients, for its neighbours, so no nodal state goes through HBM and
// one launch evaluates the residual.  A shared facet node's two traces are
// the same arithmetic on the same coefficients (row j of R V applied to the
// owning element's modes), so both sides see bitwise the same states.
//
// One warp per element; lane r owns row r of every operator product.  The
// dense V, R V, V^T, R, R^T, D_m and D_m^T are staged once per block in
// shared memory in column-major order, so the lanes' loads of one column
// are consecutive and the vector operand is a broadcast.  Between steps the
// warp synchronises with __syncwarp only.  The work is latency bound on the
// small meshes this path serves: dense products trade the sparse operators'
// index loads for a few more FMAs from shared memory.
#include "sse_device.cuh"
#include "sse_kernels.cuh"
#include "sse_ops.cuh"
#include "sse_tma.cuh"

namespace sse {

namespace {

// acc[v] += sum_c A[c * rows + r] x[v * xs + c] for v < NV
template <int NV>
__device__ __forceinline__ void col_matvec(const double *__restrict__ A, int rows, int cols, int r,
                                           const double *__restrict__ x, int xs, double (&acc)[NV]) {
#pragma unroll 4
  for (int c = 0; c < cols; ++c) {
    const double a = A[c * rows + r];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = fma(a, x[v * xs + c], acc[v]);
  }
}

// acc[v] += (A x_v)[r] for the packed operator in slot: dense, or padded
// rows (ELL) of a sparse one, A's k-th nonzero of row r at [k * rows + r]
// with its column index at the same place in OI (padding: value 0, column
// 0).  The nonzeros come in increasing column order and fma(0, x, acc) is
// acc, so both layouts give the same bits for finite x.
template <int NV>
__device__ __forceinline__ void op_matvec(const KernelArgs &ka, const double *O, const int *OI, int slot,
                                          int rows, int cols, int r, const double *__restrict__ x, int xs,
                                          double (&acc)[NV]) {
  const double *__restrict__ A = O + ka.cop_off[slot];
  const int w = ka.cop_w[slot];
  if (w == 0) {
    col_matvec<NV>(A, rows, cols, r, x, xs, acc);
    return;
  }
  const int *__restrict__ I = OI + ka.cop_i[slot];
#pragma unroll 4
  for (int k = 0; k < w; ++k) {
    const double a = A[k * rows + r];
    const int c = I[k * rows + r];
#pragma unroll
    for (int v = 0; v < NV; ++v) acc[v] = fma(a, x[v * xs + c], acc[v]);
  }
}

}  // namespace

template <int D, int NC>
__global__ void __launch_bounds__(256) std_compact_kernel(KernelArgs ka, CompactStage st) {
  extern __shared__ __align__(16) double csm[];
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const DevGeo &g = ka.geo;
  const int np = op.np, nq = op.nq, nf = op.nf, npf = op.npf, nfac = op.nfac;
  const int lane = threadIdx.x & 31, team = threadIdx.x >> 5;
  const int k = blockIdx.x * ka.epb_c + team;
  const bool live = k < ka.ne;
  const size_t kk = live ? (size_t)k : 0;
  const int nu = NC * np;

  // ---- operators (one bulk copy for the block), the element's
  // halfWLambda and mass operator (bulk copies issued by its warp), its own
  // and its neighbours' modal states (plain loads: the stage input may be
  // the caller's buffer, read only inside its bounds)
  __shared__ uint64_t cbar[1 + kMaxCompactEpb];
  double *O = csm;
  int *OI = reinterpret_cast<int *>(csm + ka.cop_doubles);
  double *E = csm + ka.cop_doubles + ka.copi_ints / 2 + (size_t)team * ka.ct_doubles;
  double *U = E + ka.ct_off[kCtU], *UQ = E + ka.ct_off[kCtUQ], *F = E + ka.ct_off[kCtF],
         *G = E + ka.ct_off[kCtG], *FF = E + ka.ct_off[kCtFF], *RQ = E + ka.ct_off[kCtRQ],
         *BM = E + ka.ct_off[kCtBM];
  double *UN = U + nu;  // face f's neighbour at UN + f nu
  const double *hwg = g.halfWLambda + kk * D * D * nq;
  const double *akg = ka.mass_wa ? ka.Ak + kk * np * np : nullptr;
  const double *HW = staged_ptr(E + ka.ct_off[kCtHW], hwg);
  const double *AK = akg ? staged_ptr(E + ka.ct_off[kCtAK], akg) : nullptr;
  uint64_t *bar_ops = &cbar[0], *bar_el = &cbar[1 + team];
  if (threadIdx.x == 0) {
    for (int t = 0; t <= ka.epb_c; ++t) mbar_init(&cbar[t], 1);
    mbar_fence_init();
    const uint32_t bytes = (uint32_t)ka.cop_doubles * 8u, ibytes = (uint32_t)ka.copi_ints * 4u;
    mbar_arrive_expect_tx(bar_ops, bytes + ibytes);
    bulk_copy_g2s(O, ka.cops, bytes, bar_ops);
    if (ibytes) bulk_copy_g2s(OI, ka.copi, ibytes, bar_ops);
  }
  __syncthreads();  // the barriers are initialised
  if (!live) return;  // no block-wide barrier follows
  if (lane == 0) {
    const uint32_t bh = (uint32_t)(D * D * nq) * 8u, ba = (uint32_t)(np * np) * 8u;
    mbar_arrive_expect_tx(bar_el, staged_span(hwg, bh) + (akg ? staged_span(akg, ba) : 0u));
    stage_slab(E + ka.ct_off[kCtHW], hwg, bh, bar_el);
    if (akg) stage_slab(E + ka.ct_off[kCtAK], akg, ba, bar_el);
  }
  // this lane's facet node: its partner (element kn, node jn), normal and BJf
  int P = 0;
  double nv[D], bjf = 0.0;
#pragma unroll
  for (int m = 0; m < D; ++m) nv[m] = 0.0;
  if (lane < nf) {
    P = __ldg(g.mapP + kk * nf + lane);
#pragma unroll
    for (int m = 0; m < D; ++m) nv[m] = __ldg(g.n_f + m + D * (lane + (size_t)nf * kk));
    bjf = __ldg(g.BJf + kk * nf + lane);
  }
  const int jn = P % nf, fj = lane < nf ? lane / npf : 0;
  // the neighbour of each face, from the lane of the face's first node
  // (every node of a face has its partner in the same element, checked on
  // the host)
  int kn[4];
#pragma unroll
  for (int f = 0; f < 4; ++f) kn[f] = __shfl_sync(0xffffffffu, P, f < nfac ? f * npf : 0) / nf;
  {
    const int total = (1 + nfac) * nu;
    const float rnu = qrcp(nu);
    const double *uin = st.uin;
    for (int t0 = 0; t0 < total; t0 += 32 * 8) {
      double v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int t = t0 + 32 * r + lane;
        v[r] = 0.0;
        if (t < total) {
          const int sl = qdiv(t, rnu), o = t - sl * nu;
          const int el = sl == 0 ? (int)kk : (sl == 1 ? kn[0] : (sl == 2 ? kn[1] : (sl == 3 ? kn[2] : kn[3])));
          v[r] = __ldg(uin + (size_t)el * nu + o);
        }
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
        const int t = t0 + 32 * r + lane;
        if (t < total) U[t] = v[r];
      }
    }
  }
  __syncwarp();
  {
    const bool ok = mbar_wait_bounded(bar_ops, 0) && mbar_wait_bounded(bar_el, 0);
    if (!__all_sync(0xffffffffu, ok)) {
      if (lane == 0) ka.flag_timeout();
      // give copies still in flight a bounded time to land before leaving
      mbar_wait_bounded(bar_ops, 0);
      mbar_wait_bounded(bar_el, 0);
      return;
    }
  }

  // ---- u_q = V u ; own and neighbour facet traces (R V) u
  if (op.has_vdm) {
    if (lane < nq) {
      double acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = 0.0;
      col_matvec<NC>(O + ka.cop_off[kCopV], nq, np, lane, U, np, acc);
#pragma unroll
      for (int e = 0; e < NC; ++e) UQ[e * nq + lane] = acc[e];
    }
  } else {
    UQ = U;  // V = I
  }
  double ui[NC], uo[NC];
#pragma unroll
  for (int e = 0; e < NC; ++e) { ui[e] = 0.0; uo[e] = 0.0; }
  if (lane < nf) {
    const double *VR = O + ka.cop_off[kCopVR];
    col_matvec<NC>(VR, nf, np, lane, U, np, ui);
    col_matvec<NC>(VR, nf, np, jn, UN + fj * nu, np, uo);
  }

  // ---- physical fluxes f_n and contracted fluxes g_m = sum_n halfWLambda[n][m] f_n
  if (lane < nq) {
    double u[NC], Fv[NC][D];
#pragma unroll
    for (int e = 0; e < NC; ++e) u[e] = UQ[e * nq + lane];
    if constexpr (NC == 1) {
#pragma unroll
      for (int n = 0; n < D; ++n) Fv[0][n] = ph.a[n] * u[0];
    } else {
      euler_flux<D>(ph, u, Fv);
    }
#pragma unroll
    for (int n = 0; n < D; ++n)
#pragma unroll
      for (int e = 0; e < NC; ++e) F[(n * NC + e) * nq + lane] = Fv[e][n];
#pragma unroll
    for (int m = 0; m < D; ++m) {
      double hw[D];
#pragma unroll
      for (int n = 0; n < D; ++n) hw[n] = HW[(m + D * n) * nq + lane];
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        double s = hw[0] * Fv[e][0];
#pragma unroll
        for (int n = 1; n < D; ++n) s = fma(hw[n], Fv[e][n], s);
        G[(m * NC + e) * nq + lane] = s;
      }
    }
  }
  // ---- numerical flux at this lane's facet node (conservative average + LF)
  double ffv[NC];
  if (lane < nf) {
    double Ft[NC][D];
    if constexpr (NC == 1) {
      two_point<D, 1>(ph, ui, uo, Ft);
    } else {
      double FL[NC][D], FR[NC][D];
      euler_flux<D>(ph, ui, FL);
      euler_flux<D>(ph, uo, FR);
#pragma unroll
      for (int e = 0; e < NC; ++e)
#pragma unroll
        for (int n = 0; n < D; ++n) Ft[e][n] = 0.5 * (FL[e][n] + FR[e][n]);
    }
    double a = 0.0;
    if (ph.nflux == 0) a = ph.half_lambda * wave_speed<D, NC>(ph, ui, uo, nv);
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      double fn = 0.0;
#pragma unroll
      for (int m = 0; m < D; ++m) fn = fma(Ft[e][m], nv[m], fn);
      ffv[e] = (ph.nflux == 0) ? fma(a, ui[e] - uo[e], fn) : fn;
    }
  }
  __syncwarp();

  // ---- r_q = sum_m D_m^T g_m - sum_{n,m} halfWLambda[n][m] (D_m f_n)
  double r[NC];
#pragma unroll
  for (int e = 0; e < NC; ++e) r[e] = 0.0;
  if (lane < nq) {
#pragma unroll
    for (int m = 0; m < D; ++m) {
      double a1[NC], a2[D * NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) a1[e] = 0.0;
#pragma unroll
      for (int v = 0; v < D * NC; ++v) a2[v] = 0.0;
      op_matvec<NC>(ka, O, OI, kCopDT + m, nq, nq, lane, G + m * NC * nq, nq, a1);
      op_matvec<D * NC>(ka, O, OI, kCopD + m, nq, nq, lane, F, nq, a2);
#pragma unroll
      for (int e = 0; e < NC; ++e) r[e] += a1[e];
#pragma unroll
      for (int n = 0; n < D; ++n) {
        const double hw = HW[(m + D * n) * nq + lane];
#pragma unroll
        for (int e = 0; e < NC; ++e) r[e] = fma(-hw, a2[n * NC + e], r[e]);
      }
    }
  }
  // ---- f_f -= sum_n halfN_n (R f_n) ; f_f .*= BJf
  if (lane < nf) {
    double a3[D * NC];
#pragma unroll
    for (int v = 0; v < D * NC; ++v) a3[v] = 0.0;
    op_matvec<D * NC>(ka, O, OI, kCopR, nf, nq, lane, F, nq, a3);
#pragma unroll
    for (int n = 0; n < D; ++n) {
      const double halfN = 0.5 * nv[n];
#pragma unroll
      for (int e = 0; e < NC; ++e) ffv[e] -= a3[n * NC + e] * halfN;
    }
#pragma unroll
    for (int e = 0; e < NC; ++e) FF[e * nf + lane] = ffv[e] * bjf;
  }
  __syncwarp();
  // ---- r_q -= R^T f_f
  if (lane < nq) {
    double a4[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) a4[e] = 0.0;
    op_matvec<NC>(ka, O, OI, kCopRT, nq, nf, lane, FF, nf, a4);
#pragma unroll
    for (int e = 0; e < NC; ++e) RQ[e * nq + lane] = r[e] - a4[e];
  }
  __syncwarp();
  // ---- V^T r_q, then the mass solve
  if (lane < np) {
    double bm[NC];
    if (op.has_vdm) {
#pragma unroll
      for (int e = 0; e < NC; ++e) bm[e] = 0.0;
      col_matvec<NC>(O + ka.cop_off[kCopVT], np, nq, lane, RQ, nq, bm);
    } else {
#pragma unroll
      for (int e = 0; e < NC; ++e) bm[e] = RQ[e * nq + lane];
    }
#pragma unroll
    for (int e = 0; e < NC; ++e) BM[e * np + lane] = bm[e];
  }
  __syncwarp();
  if (lane >= np) return;
  double x[NC];
  if (ka.mass_wa) {
    // the element's weight-adjusted mass operator (n_p x n_p, column-major)
#pragma unroll
    for (int e = 0; e < NC; ++e) x[e] = 0.0;
    col_matvec<NC>(AK, np, np, lane, BM, np, x);
  } else {
    const double w = g.WJinv[kk * nq + lane];
#pragma unroll
    for (int e = 0; e < NC; ++e) x[e] = BM[e * np + lane] * w;
  }

  // ---- the residual, or the Runge-Kutta stage it feeds
#pragma unroll
  for (int e = 0; e < NC; ++e) {
    const size_t idx = kk * nu + (size_t)e * np + lane;
    const double kx = x[e];
    if (!isfinite(kx)) ka.flag_nonphysical();
    switch (st.mode) {
      case kCompactResidual:
        st.out[idx] = kx;
        break;
      case kCompactRK4:
        st.acc[idx] = st.first ? kx : st.acc[idx] + st.w * kx;
        st.out[idx] = st.ubase[idx] + st.c * kx;
        break;
      case kCompactRK4Final:
        st.out[idx] = st.ubase[idx] + st.c * (st.acc[idx] + kx);
        break;
      default: {
        const double t = st.first ? st.dt * kx : st.a * st.acc[idx] + st.dt * kx;
        st.acc[idx] = t;
        st.out[idx] = st.uin[idx] + st.b * t;
      }
    }
  }
}

// column a of V: V applied to the a-th unit vector by the sum-factorised (or
// dense) product every other kernel uses
template <int D>
__global__ void __launch_bounds__(128) dense_vdm_kernel(KernelArgs ka, double *out) {
  extern __shared__ double vsm[];
  const Layout &L = ka.layA;
  double *X = vsm + L.off[0], *Y = vsm + L.off[1], *Z = vsm + L.off[2], *W = vsm + L.off[3];
  const int a = blockIdx.x, np = ka.op.np, nq = ka.op.nq;
  for (int t = threadIdx.x; t < np; t += blockDim.x) X[t] = t == a ? 1.0 : 0.0;
  __syncthreads();
  vdm_mul<double, D, 1>(ka.op, X, Y, Z, W, threadIdx.x, blockDim.x);
  for (int i = threadIdx.x; i < nq; i += blockDim.x) out[(size_t)a * nq + i] = Y[i];
}

#define SSE_COMPACT_DISPATCH(CALL)                                          \
  if (ka.op.d == 2 && ka.op.nc == 1) { constexpr int D = 2, NC = 1; CALL; }   \
  else if (ka.op.d == 2 && ka.op.nc == 4) { constexpr int D = 2, NC = 4; CALL; } \
  else if (ka.op.d == 3 && ka.op.nc == 1) { constexpr int D = 3, NC = 1; CALL; } \
  else if (ka.op.d == 3 && ka.op.nc == 5) { constexpr int D = 3, NC = 5; CALL; } \
  else return cudaErrorInvalidValue;

cudaError_t sse_set_smem_limit_compact(const KernelArgs &ka, size_t bytes) {
  cudaError_t e = cudaSuccess;
  SSE_COMPACT_DISPATCH((e = cudaFuncSetAttribute((const void *)std_compact_kernel<D, NC>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes)));
  return e;
}

cudaError_t launch_std_compact(const KernelArgs &ka, const CompactStage &st, cudaStream_t s) {
  const int grid = (ka.ne + ka.epb_c - 1) / ka.epb_c;
  const size_t sm = ((size_t)ka.cop_doubles + ka.copi_ints / 2 + (size_t)ka.epb_c * ka.ct_doubles) * sizeof(double);
  SSE_COMPACT_DISPATCH((std_compact_kernel<D, NC><<<grid, 32 * ka.epb_c, sm, s>>>(ka, st)));
  return cudaGetLastError();
}

cudaError_t launch_dense_vdm(const KernelArgs &ka, double *out, cudaStream_t s) {
  const size_t sm = (size_t)ka.layA.team_doubles * sizeof(double);
  cudaError_t e;
  if (ka.op.d == 2) {
    if ((e = cudaFuncSetAttribute((const void *)dense_vdm_kernel<2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sm)))
      return e;
    dense_vdm_kernel<2><<<ka.op.np, 128, sm, s>>>(ka, out);
  } else {
    if ((e = cudaFuncSetAttribute((const void *)dense_vdm_kernel<3>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)sm)))
      return e;
    dense_vdm_kernel<3><<<ka.op.np, 128, sm, s>>>(ka, out);
  }
  return cudaGetLastError();
}

#undef SSE_COMPACT_DISPATCH

}  // namespace sse
