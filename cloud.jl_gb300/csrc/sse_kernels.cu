// sse_kernels.cu -- sm_103a kernels of the semi-discrete residual.
//
// Work decomposition: a CTA holds EPB elements; each element is handled by a
// team of TPE = blockDim.x / EPB threads that keeps every per-element array
// (states, fluxes, partial sums, sum-factorisation stages) in shared memory.
// Global memory is touched once per array per phase: the element's modal
// coefficients, its metric terms and, in phase B, the neighbours' facet
// states gathered through mapP.  Pair sums are accumulated in two passes
// (per-pair contributions, then a fixed-order per-node reduction), so the
// result is deterministic run to run.
//
// Phase A  nodal_values_kernel     nodal_values! / entropy_projection!
//          (standard_form_first_order.jl:1-14, flux_differencing_form.jl:190-292)
// Phase B  fd_time_derivative_kernel   time_derivative! FD (flux_differencing_form.jl:294-347)
//          std_time_derivative_kernel  time_derivative! StandardForm (standard_form_first_order.jl:16-63)
#include "sse_device.cuh"
#include "sse_kernels.cuh"
#include "sse_tma.cuh"
#include "sse_ops.cuh"

namespace sse {

// ---------------------------------------------------------------------------
// Phase A: nodal_values!
// ---------------------------------------------------------------------------
template <int D, int NC>
__global__ void __launch_bounds__(256) nodal_values_kernel(KernelArgs ka) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Layout &L = ka.layA;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  double *base = smem + (size_t)team * L.team_doubles;
  double *X = base + L.off[0], *Y = base + L.off[1], *Z = base + L.off[2], *Wb = base + L.off[3],
         *F = base + L.off[4];
  const int np = op.np, nq = op.nq, nf = op.nf;
  const double *uk = ka.u + (size_t)kk * NC * np;
  const bool project = ka.project_entropy;

  for (int t = lane; t < NC * np; t += tpe) X[t] = uk[t];
  __syncthreads();
  vdm_mul<double, D, NC>(op, X, Y, Z, Wb, lane, tpe);  // Y = u_q = V u

  double *uq_out = ka.u_q + (size_t)kk * NC * nq;
  double *uf_out = ka.u_f + (size_t)kk * NC * nf;
  if constexpr (NC > 1) {
    if (project) {
      const Physics &ph = ka.ph;
      const double *WJ = ka.geo.WJ + (size_t)kk * nq;
      // w_q = WJ .* c2e(u_q)   (entropy_projection!, flux_differencing_form.jl:229-235)
      for (int i = lane; i < nq; i += tpe) {
        double ui[NC], wi[NC];
#pragma unroll
        for (int e = 0; e < NC; ++e) ui[e] = Y[e * nq + i];
        if (!(ui[0] > 0.0)) ka.flag_nonphysical();
        cons_to_entropy_fast<D>(ph.gamma, ph.gm1, ph.igm1, ui, wi, op.math_tab);
        double s = op.has_vdm ? WJ[i] : 1.0;
#pragma unroll
        for (int e = 0; e < NC; ++e) X[e * nq + i] = wi[e] * s;
      }
      __syncthreads();
      if (op.has_vdm) {
        // X holds WJ w_q (NC x nq): w = V^T (WJ w_q); mass solve; w_q = V w
        double *Wm = F;  // NC x np modal scratch (F is large enough, see layout)
        vdm_tmul<double, D, NC>(op, X, Wm, Z, Wb, lane, tpe);
        mass_solve<double, D, NC>(op, ka.geo.JinvW + (size_t)kk * nq, nullptr, 1, Wm, X, Z, Wb, lane, tpe,
                                  ka.Ak ? ka.Ak + (size_t)kk * op.np * op.np : nullptr);
        vdm_mul<double, D, NC>(op, Wm, X, Z, Wb, lane, tpe);  // X = w_q (projected)
        // u_q = e2c(w_q)
        for (int i = lane; i < nq; i += tpe) {
          double wi[NC], ui[NC];
#pragma unroll
          for (int e = 0; e < NC; ++e) wi[e] = X[e * nq + i];
          entropy_to_cons_fast<D>(ph.gamma, ph.gm1, ph.igm1, ph.log_gm1, wi, ui, op.math_tab);
#pragma unroll
          for (int e = 0; e < NC; ++e) {
            if (live) store_state<NC>(ka, ka.u_q, ka.u_qf, (size_t)kk * NC * nq + e * nq + i, e, ui[e]);
            if (!(ui[0] > 0.0) || !isfinite(ui[e])) ka.flag_nonphysical();
          }
        }
      } else {
        // nodal: u_q stays u; X = w_q
        for (int t = lane; t < NC * nq; t += tpe)
          if (live) store_state<NC>(ka, ka.u_q, ka.u_qf, (size_t)kk * NC * nq + t, t / nq, Y[t]);
      }
      // w_f = R w_q ; u_f = e2c(w_f)
      csr_mul<double, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_val, X, F, lane, tpe);
      __syncthreads();
      for (int j = lane; j < nf; j += tpe) {
        double wi[NC], ui[NC];
#pragma unroll
        for (int e = 0; e < NC; ++e) wi[e] = F[e * nf + j];
        entropy_to_cons_fast<D>(ph.gamma, ph.gm1, ph.igm1, ph.log_gm1, wi, ui, op.math_tab);
#pragma unroll
        for (int e = 0; e < NC; ++e) {
          if (live) store_state<NC>(ka, ka.u_f, ka.u_ff, (size_t)kk * NC * nf + e * nf + j, e, ui[e]);
          if (!(ui[0] > 0.0) || !isfinite(ui[e])) ka.flag_nonphysical();
        }
      }
      return;
    }
  }
  // no projection: u_q = V u; u_f = R u_q
  for (int t = lane; t < NC * nq; t += tpe)
    if (live) uq_out[t] = Y[t];
  csr_mul<double, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_val, Y, F, lane, tpe);
  __syncthreads();
  for (int t = lane; t < NC * nf; t += tpe)
    if (live) uf_out[t] = F[t];
}

// ---------------------------------------------------------------------------
// numerical flux at the element's facet nodes, scaled by BJf
// (numerical_flux!, ConservationLaws.jl:75-128; lmul!(BJf[k], f_f))
// ---------------------------------------------------------------------------
template <int D, int NC>
__device__ void facet_flux(const KernelArgs &ka, int kk, const double *uf, double *ff, int ec,
                           int lane, int tpe, const double *prim_f) {
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const int nf = op.nf;
  for (int j = lane; j < nf; j += tpe) {
    int P = ka.geo.mapP[(size_t)kk * nf + j];
    int jn = P % nf, kn = P / nf;
    double ui[NC], uo[NC], n[D], F[NC][D];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      ui[e] = uf[e * nf + j];
      uo[e] = ka.u_f[((size_t)kn * NC + e) * nf + jn];
    }
#pragma unroll
    for (int m = 0; m < D; ++m) n[m] = ka.geo.n_f[m + D * (j + (size_t)nf * kk)];
    if constexpr (NC > 1) {
      if (ec && prim_f) {
        // entropy-conservative flux . n from per-node primitives, plus LF
        const double *Pi = prim_f + (size_t)j * (3 + D);
        double Po[3 + D], out[NC];
        euler_prim_fast<D>(ph.gm1, uo, Po);
        ec_flux_dot<D>(ph.igm1, Pi, Po, n, out);
        double a = 0.0;
        if (ph.nflux == 0) {
          double vni = 0.0, vno = 0.0;
#pragma unroll
          for (int m = 0; m < D; ++m) { vni = fma(Pi[3 + m], n[m], vni); vno = fma(Po[3 + m], n[m], vno); }
          double ci = sqrt(ph.gamma * Pi[1] * sse_rcp(Pi[0]));
          double co = sqrt(ph.gamma * Po[1] * sse_rcp(Po[0]));
          a = ph.half_lambda * (fmax(fabs(vni), fabs(vno)) + fmax(ci, co));
        }
        double bjf = ka.geo.BJf[(size_t)kk * nf + j];
#pragma unroll
        for (int e = 0; e < NC; ++e) {
          double fs = (ph.nflux == 0) ? fma(a, ui[e] - uo[e], out[e]) : out[e];
          ff[e * nf + j] = fs * bjf;
        }
        continue;
      }
    }
    Physics ph2 = ph;
    ph2.ec = ec;
    two_point<D, NC>(ph2, ui, uo, F);
    double a = 0.0;
    if (ph.nflux == 0) a = ph.half_lambda * wave_speed<D, NC>(ph, ui, uo, n);
    double bjf = ka.geo.BJf[(size_t)kk * nf + j];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      double fn = 0.0;
#pragma unroll
      for (int m = 0; m < D; ++m) fn = fma(F[e][m], n[m], fn);
      double fs = (ph.nflux == 0) ? fma(a, ui[e] - uo[e], fn) : fn;
      ff[e * nf + j] = fs * bjf;
    }
  }
}

// ---------------------------------------------------------------------------
// Mixed-form phase A (modal V): the entropy projection with its operator
// arithmetic in FP32.  With w_ref the entropy variables of the constant
// reference state, the projection P = V M^-1 V^T diag(W J) is linear, so
//   P w = w_ref P(1) + P(w - w_ref):
// P(1) and R P(1) are precomputed per element in FP64, and P is applied in
// FP32 only to the perturbation w - w_ref, which is small where the flow is
// near the reference state.  V u runs in FP32 on u - u_ref, and both
// entropy-variable maps run in FP32 on perturbations (cons_to_entropy_pert,
// entropy_to_cons_pert), so the kernel has almost no FP64 work.
// ---------------------------------------------------------------------------
template <int D, int NC>
__global__ void __launch_bounds__(256) nodal_values_mixed_kernel(KernelArgs ka) {
  static_assert(NC == D + 2, "mixed form of the Euler entropy projection");
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const Layout &L = ka.layAm;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq, nf = op.nf;
  double *base = smem + (size_t)team * L.team_doubles;
  float *fb = reinterpret_cast<float *>(base + L.off[4]);
  float *Af = fb + L.off[5], *Bf = fb + L.off[6], *Cf = fb + L.off[7], *Zf = fb + L.off[8],
        *Wf = fb + L.off[9];

  // u - u_ref in modal coefficients (only the constant mode changes), FP32;
  // u_q = u_ref + V (u - u_ref) with V applied in FP32
  const double *uk = ka.u + (size_t)kk * NC * np;
  for (int t = lane; t < NC * np; t += tpe) {
    const int e = t / np, l = t - e * np;
    Cf[t] = (float)(l == ph.mode0 ? uk[t] - ph.u_ref_modal[e] : uk[t]);
  }
  __syncthreads();
  vdm_mul<float, D, NC>(op, Cf, Bf, Zf, Wf, lane, tpe);
  const EntropyRefF &cr = ph.cref;
  // x' = W J (c2e(u_q) - w_ref)
  for (int i = lane; i < nq; i += tpe) {
    float ui[NC], wi[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) ui[e] = Bf[e * nq + i];
    if (!(cr.rho_ref + ui[0] > 0.f)) ka.flag_nonphysical();
    cons_to_entropy_pert<D>(cr, ui, wi);
    const float wj = ka.geo.WJf[(size_t)kk * nq + i];
#pragma unroll
    for (int e = 0; e < NC; ++e) Af[e * nq + i] = wj * wi[e];
  }
  __syncthreads();
  vdm_tmul<float, D, NC>(op, Af, Cf, Zf, Wf, lane, tpe);                               // V^T x'
  mass_solve<float, D, NC>(op, ka.geo.JinvWf + (size_t)kk * nq, nullptr, 1, Cf, Af, Zf, Wf, lane, tpe, ka.Akf ? ka.Akf + (size_t)kk * op.np * op.np : nullptr);
  vdm_mul<float, D, NC>(op, Cf, Bf, Zf, Wf, lane, tpe);                                // w'_q
  csr_mul<float, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_valf, Bf, Af, lane, tpe);        // w'_f
  __syncthreads();
  const float *P1m1 = ka.geo.P1m1f + (size_t)kk * nq, *RP1m1 = ka.geo.RP1m1f + (size_t)kk * nf;
  // w - w_ref = w_ref (P(1) - 1) + P(w - w_ref) at the volume and facet
  // nodes; u' = e2c(w) - u_ref, stored as the FP32 states of phase B
  for (int t = lane; t < nq + nf; t += tpe) {
    const bool vol = t < nq;
    const int r = vol ? t : t - nq;
    const float p1m1 = vol ? P1m1[r] : RP1m1[r];
    const float *src = vol ? Bf + r : Af + r;
    const int stride = vol ? nq : nf;
    float wi[NC], ui[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) wi[e] = fmaf(cr.w_ref[e], p1m1, src[e * stride]);
    entropy_to_cons_pert<D>(cr, wi, ui);
    const size_t o = (size_t)kk * NC * (vol ? nq : nf) + r;
    float *dst = vol ? ka.u_qf : ka.u_ff;
    if (!(cr.rho_ref + ui[0] > 0.f)) ka.flag_nonphysical();
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      if (live) dst[o + (size_t)e * stride] = ui[e];
      if (!isfinite(ui[e])) ka.flag_nonphysical();
    }
  }
}

// The entropy projection of the constant function 1 on every element,
// P(1) = V M^-1 V^T (W J) with the weight-adjusted inverse, and R P(1).
template <int D>
__global__ void __launch_bounds__(256) projection_of_one_kernel(KernelArgs ka, double *P1, double *RP1) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Layout &L = ka.layP1;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int nq = op.nq, nf = op.nf;
  double *base = smem + (size_t)team * L.team_doubles;
  double *X = base + L.off[0], *Y = base + L.off[1], *Z = base + L.off[2], *Wb = base + L.off[3],
         *F = base + L.off[4];
  for (int t = lane; t < nq; t += tpe) X[t] = ka.geo.WJ[(size_t)kk * nq + t];
  __syncthreads();
  vdm_tmul<double, D, 1>(op, X, F, Z, Wb, lane, tpe);
  mass_solve<double, D, 1>(op, ka.geo.JinvW + (size_t)kk * nq, nullptr, 1, F, X, Z, Wb, lane, tpe);
  vdm_mul<double, D, 1>(op, F, Y, Z, Wb, lane, tpe);
  csr_mul<double, 1>(nf, nq, op.R_ptr, op.R_idx, op.R_val, Y, F, lane, tpe);
  __syncthreads();
  if (live) {
    for (int t = lane; t < nq; t += tpe) P1[(size_t)kk * nq + t] = Y[t];
    for (int t = lane; t < nf; t += tpe) RP1[(size_t)kk * nf + t] = F[t];
  }
}

// ---------------------------------------------------------------------------
// Phase B, FluxDifferencingForm
// ---------------------------------------------------------------------------
template <int D, int NC>
__global__ void __launch_bounds__(256) fd_time_derivative_kernel(KernelArgs ka) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const Layout &L = ka.layB;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq, nf = op.nf, nfac = op.nfac, npf = op.npf;
  const float rnpf = qrcp(npf > 0 ? npf : 1);
  double *base = smem + (size_t)team * L.team_doubles;
  double *uq = base + L.off[0], *uf = base + L.off[1], *ff = base + L.off[2], *rq = base + L.off[3],
         *diff = base + L.off[4], *Lam = base + L.off[5], *hnq = base + L.off[6],
         *prim = base + L.off[7];

  // stage the element's data
  const double *uqg = ka.u_q + (size_t)kk * NC * nq;
  const double *ufg = ka.u_f + (size_t)kk * NC * nf;
  for (int t = lane; t < NC * nq; t += tpe) uq[t] = uqg[t];
  for (int t = lane; t < NC * nf; t += tpe) uf[t] = ufg[t];
  const double *Lg = ka.geo.Lambda_q + (size_t)kk * nq * D * D;
  for (int t = lane; t < nq * D * D; t += tpe) Lam[t] = Lg[t];
  const double *Hg = ka.geo.halfnJq + (size_t)kk * D * nfac * nq;
  if (op.nfp > 0)
    for (int t = lane; t < D * nfac * nq; t += tpe) hnq[t] = Hg[t];
  __syncthreads();

  const int ec = ph.ec;
  // per-node primitive quantities for the Euler EC flux: [rho, p, beta, V_1..V_D]
  const int PS = 3 + D;
  if constexpr (NC > 1) {
    if (ec) {
      for (int i = lane; i < nq + nf; i += tpe) {
        double u[NC];
#pragma unroll
        for (int e = 0; e < NC; ++e) u[e] = (i < nq) ? uq[e * nq + i] : uf[e * nf + (i - nq)];
        euler_prim_fast<D>(ph.gm1, u, prim + (size_t)i * PS);
      }
      __syncthreads();
    }
  }
  facet_flux<D, NC>(ka, kk, uf, ff, ec, lane, tpe, (NC > 1 && ec) ? prim + (size_t)nq * PS : nullptr);

  // volume flux differencing (flux_difference!, flux_differencing_form.jl:
  // 37-75), one flux per unique pair, over chunks of at most CH pairs so the
  // per-pair buffer stays small: pass 1 writes each pair's contribution,
  // pass 2 adds them to r_q at both nodes in ascending pair order
  // (deterministic; each node keeps a cursor into its incidence list).  For
  // the EC flux the metric vector G[n] = sum_m S_m (Lambda_i + Lambda_j)[m, n]
  // is formed first and contracted inside the flux.
  const int CH = ka.fd_chunk;
  int cur[kMaxNodeSlots];
#pragma unroll
  for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
    const int i = lane + sl * tpe;
    cur[sl] = i < nq ? op.vp_inc_ptr[i] : 0;
    if (i < nq && CH < op.nvp)
      for (int e = 0; e < NC; ++e) rq[e * nq + i] = 0.0;
  }
  for (int c0 = 0; c0 < op.nvp; c0 += CH) {
    const int c1 = min(op.nvp, c0 + CH);
    // with all pairs in one chunk, the lanes that also computed an interface
    // flux take vp_split pairs each from the front of the list and the other
    // lanes share the rest (which thread computes a pair does not change
    // the sums, taken in pair order)
    const bool split = ka.vp_split > 0 && c0 == 0 && c1 == op.nvp;
    const int pfirst = split ? (lane < nf ? lane : ka.vp_split * nf + (lane - nf)) : c0 + lane;
    const int pstep = split ? (lane < nf ? nf : tpe - nf) : tpe;
    const int plast = split ? (lane < nf ? ka.vp_split * nf : c1) : c1;
    for (int pidx = pfirst; pidx < plast; pidx += pstep) {
      int ij = op.vp_ij[pidx];
      int i = ij & 0xffff, j = ij >> 16;
      double *dp = diff + (size_t)(pidx - c0) * NC;
      if constexpr (NC > 1) {
        if (ec) {
          double G[D];
#pragma unroll
          for (int n = 0; n < D; ++n) G[n] = 0.0;
#pragma unroll
          for (int m = 0; m < D; ++m) {
            const double Sm = op.vp_Sh[pidx * D + m];
            if (Sm == 0.0) continue;
#pragma unroll
            for (int n = 0; n < D; ++n)
              G[n] = fma(Sm, Lam[i + nq * (m + D * n)] + Lam[j + nq * (m + D * n)], G[n]);
          }
          ec_flux_dot_half<D>(ph.igm1, ph.ilm_q, prim + (size_t)i * PS, prim + (size_t)j * PS, G, dp);
          continue;
        }
      }
      double F[NC][D];
      if constexpr (NC > 1) {
        {
          double ui[NC], uj[NC];
#pragma unroll
          for (int e = 0; e < NC; ++e) { ui[e] = uq[e * nq + i]; uj[e] = uq[e * nq + j]; }
          two_point<D, NC>(ph, ui, uj, F);
        }
      } else {
        double ui[1] = {uq[i]}, uj[1] = {uq[j]};
        two_point<D, NC>(ph, ui, uj, F);
      }
      double out[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) out[e] = 0.0;
#pragma unroll
      for (int m = 0; m < D; ++m) {
        double Sm = op.vp_S[pidx * D + m];
        if (Sm == 0.0) continue;
        double Lij[D];
#pragma unroll
        for (int n = 0; n < D; ++n) Lij[n] = Lam[i + nq * (m + D * n)] + Lam[j + nq * (m + D * n)];
#pragma unroll
        for (int e = 0; e < NC; ++e) {
          double Fm = 0.0;
#pragma unroll
          for (int n = 0; n < D; ++n) Fm = fma(Lij[n], F[e][n], Fm);
          out[e] = fma(Sm, Fm, out[e]);
        }
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) dp[e] = out[e];
    }
    __syncthreads();
    // r_q[i] += -diff if i is the pair's first node, +diff otherwise
    if (CH >= op.nvp) {
      // one chunk: each node sums its whole incidence list
      for (int i = lane; i < nq; i += tpe) {
        double acc[NC];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = 0.0;
        for (int q = op.vp_inc_ptr[i]; q < op.vp_inc_ptr[i + 1]; ++q) {
          const int inc = op.vp_inc[q];
          const double sgn = (inc & 1) ? -1.0 : 1.0;
          const double *dp = diff + (size_t)(inc >> 1) * NC;
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] = fma(sgn, dp[e], acc[e]);
        }
#pragma unroll
        for (int e = 0; e < NC; ++e) rq[e * nq + i] = acc[e];
      }
      __syncthreads();
      continue;
    }
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int i = lane + sl * tpe;
      if (i >= nq) continue;
      double acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = rq[e * nq + i];
      int q = cur[sl];
      const int qe = op.vp_inc_ptr[i + 1];
      for (; q < qe; ++q) {
        const int inc = op.vp_inc[q];
        const int pidx = inc >> 1;
        if (pidx >= c1) break;
        const double sgn = (inc & 1) ? -1.0 : 1.0;
        const double *dp = diff + (size_t)(pidx - c0) * NC;
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = fma(sgn, dp[e], acc[e]);
      }
      cur[sl] = q;
#pragma unroll
      for (int e = 0; e < NC; ++e) rq[e * nq + i] = acc[e];
    }
    __syncthreads();
  }

  // facet correction (facet_correction!, flux_differencing_form.jl:126-168),
  // chunked the same way; each chunk's sum is subtracted from r_q / f_f
  if (op.nfp > 0) {
    const double *hnf = ka.geo.halfnJf + (size_t)kk * D * nf;
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int t = lane + sl * tpe;
      cur[sl] = t < nq ? op.fp_q_ptr[t] : (t < nq + nf ? op.fp_f_ptr[t - nq] : 0);
    }
    for (int c0 = 0; c0 < op.nfp; c0 += CH) {
      const int c1 = min(op.nfp, c0 + CH);
      for (int pidx = c0 + lane; pidx < c1; pidx += tpe) {
        int ij = op.fp_ij[pidx];
        int i = ij & 0xffff, j = ij >> 16;
        int f = qdiv(j, rnpf);
        double *dp = diff + (size_t)(pidx - c0) * NC;
        if constexpr (NC > 1) {
          if (ec) {
            const double Cij = op.fp_Ch[pidx];
            double G[D];
#pragma unroll
            for (int m = 0; m < D; ++m) G[m] = Cij * (hnf[m + D * j] + hnq[m + D * (f + nfac * i)]);
            ec_flux_dot_half<D>(ph.igm1, ph.ilm_q, prim + (size_t)i * PS, prim + (size_t)(nq + j) * PS, G, dp);
            continue;
          }
        }
        double F[NC][D];
        if constexpr (NC > 1) {
          {
            double ui[NC], uj[NC];
#pragma unroll
            for (int e = 0; e < NC; ++e) { ui[e] = uq[e * nq + i]; uj[e] = uf[e * nf + j]; }
            two_point<D, NC>(ph, ui, uj, F);
          }
        } else {
          double ui[1] = {uq[i]}, uj[1] = {uf[j]};
          two_point<D, NC>(ph, ui, uj, F);
        }
        double nJ[D];
#pragma unroll
        for (int m = 0; m < D; ++m) nJ[m] = hnf[m + D * j] + hnq[m + D * (f + nfac * i)];
        double Cij = op.fp_C[pidx];
#pragma unroll
        for (int e = 0; e < NC; ++e) {
          double Fn = 0.0;
#pragma unroll
          for (int m = 0; m < D; ++m) Fn = fma(nJ[m], F[e][m], Fn);
          dp[e] = Cij * Fn;
        }
      }
      __syncthreads();
      if (CH >= op.nfp) {
        // one chunk: each node sums its whole incidence list
        for (int t = lane; t < nq + nf; t += tpe) {
          double acc[NC];
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] = 0.0;
          const bool vol = t < nq;
          const int r = vol ? t : t - nq;
          const int *ptr = vol ? op.fp_q_ptr : op.fp_f_ptr;
          const int *lst = vol ? op.fp_q : op.fp_f;
          for (int q = ptr[r]; q < ptr[r + 1]; ++q) {
            const double *dp = diff + (size_t)lst[q] * NC;
#pragma unroll
            for (int e = 0; e < NC; ++e) acc[e] += dp[e];
          }
          double *dst = vol ? rq + r : ff + r;
          const int stride = vol ? nq : nf;
#pragma unroll
          for (int e = 0; e < NC; ++e) dst[e * stride] -= acc[e];
        }
        __syncthreads();
        continue;
      }
#pragma unroll
      for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
        const int t = lane + sl * tpe;
        if (t >= nq + nf) continue;
        double acc[NC];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = 0.0;
        const bool vol = t < nq;
        const int r = vol ? t : t - nq;
        const int *lst = vol ? op.fp_q : op.fp_f;
        const int qe = vol ? op.fp_q_ptr[r + 1] : op.fp_f_ptr[r + 1];
        int q = cur[sl];
        for (; q < qe; ++q) {
          const int pidx = lst[q];
          if (pidx >= c1) break;
          const double *dp = diff + (size_t)(pidx - c0) * NC;
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] += dp[e];
        }
        cur[sl] = q;
        double *dst = vol ? rq + r : ff + r;
        const int stride = vol ? nq : nf;
#pragma unroll
        for (int e = 0; e < NC; ++e) dst[e * stride] -= acc[e];
      }
      __syncthreads();
    }
  }

  // r_q -= R^T f_f
  rt_apply<double, NC>(op, op.Rt_val, ff, lane, tpe, [&](int t, double v) { rq[t] -= v; });
  __syncthreads();

  // dudt = V^T r_q ; mass solve  (the pair buffer is free now: it holds the
  // modal and nodal buffers and the sum-factorisation scratch)
  double *Xm = diff, *Yq = diff + (size_t)NC * np;
  double *Z = Yq + (size_t)NC * nq;
  double *Wb = Z + ka.vdm_zsz;
  vdm_tmul<double, D, NC>(op, rq, Xm, Z, Wb, lane, tpe);
  mass_solve<double, D, NC>(op, ka.geo.JinvW ? ka.geo.JinvW + (size_t)kk * nq : nullptr,
                    ka.geo.WJinv ? ka.geo.WJinv + (size_t)kk * nq : nullptr, ka.mass_wa, Xm, Yq,
                    Z, Wb, lane, tpe, ka.Ak ? ka.Ak + (size_t)kk * op.np * op.np : nullptr);
  double *out = ka.dudt + (size_t)kk * NC * np;
  if (live)
    for (int t = lane; t < NC * np; t += tpe) {
      out[t] = Xm[t];
      if (!isfinite(Xm[t])) ka.flag_nonphysical();
    }
}

// ---------------------------------------------------------------------------
// Phase B, StandardForm with ReferenceOperators
// ---------------------------------------------------------------------------
template <int D, int NC>
__global__ void __launch_bounds__(256) std_time_derivative_kernel(KernelArgs ka) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const Layout &L = ka.layB;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq, nf = op.nf;
  double *base = smem + (size_t)team * L.team_doubles;
  double *uq = base + L.off[0], *uf = base + L.off[1], *ff = base + L.off[2], *rq = base + L.off[3],
         *fq = base + L.off[4], *tmp = base + L.off[5], *tmp2 = base + L.off[6], *Z = base + L.off[8],
         *Wb = base + L.off[9];

  const double *uqg = ka.u_q + (size_t)kk * NC * nq;
  const double *ufg = ka.u_f + (size_t)kk * NC * nf;
  for (int t = lane; t < NC * nq; t += tpe) uq[t] = uqg[t];
  for (int t = lane; t < NC * nf; t += tpe) uf[t] = ufg[t];
  __syncthreads();
  // f_q[n][e][i] = physical flux
  for (int i = lane; i < nq; i += tpe) {
    if constexpr (NC == 1) {
#pragma unroll
      for (int n = 0; n < D; ++n) fq[n * nq + i] = ph.a[n] * uq[i];
    } else {
      double u[NC], F[NC][D];
#pragma unroll
      for (int e = 0; e < NC; ++e) u[e] = uq[e * nq + i];
      euler_flux<D>(ph, u, F);
#pragma unroll
      for (int n = 0; n < D; ++n)
#pragma unroll
        for (int e = 0; e < NC; ++e) fq[(n * NC + e) * nq + i] = F[e][n];
    }
  }
  // numerical flux with the conservative two-point flux; not yet scaled by BJf
  {
    const int nff = nf;
    for (int j = lane; j < nff; j += tpe) {
      int P = ka.geo.mapP[(size_t)kk * nf + j];
      int jn = P % nf, kn = P / nf;
      double ui[NC], uo[NC], n[D], F[NC][D];
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        ui[e] = uf[e * nf + j];
        uo[e] = ka.u_f[((size_t)kn * NC + e) * nf + jn];
      }
#pragma unroll
      for (int m = 0; m < D; ++m) n[m] = ka.geo.n_f[m + D * (j + (size_t)nf * kk)];
      Physics ph2 = ph;
      ph2.ec = 0;
      ph2.chandrashekar = 0;
      two_point<D, NC>(ph2, ui, uo, F);
      double a = 0.0;
      if (ph.nflux == 0) a = ph.half_lambda * wave_speed<D, NC>(ph, ui, uo, n);
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        double fn = 0.0;
#pragma unroll
        for (int m = 0; m < D; ++m) fn = fma(F[e][m], n[m], fn);
        ff[e * nf + j] = (ph.nflux == 0) ? fma(a, ui[e] - uo[e], fn) : fn;
      }
    }
  }
  for (int t = lane; t < NC * nq; t += tpe) rq[t] = 0.0;
  __syncthreads();
  const double *hwl = ka.geo.halfWLambda + (size_t)kk * nq * D * D;
  for (int n = 0; n < D; ++n) {
    const double *fn_ = fq + (size_t)n * NC * nq;
    for (int m = 0; m < D; ++m) {
      const double *hw = hwl + nq * (m + D * n);
      // tmp = halfWLambda .* f_n ; tmp2 = D_m f_n
      for (int t = lane; t < NC * nq; t += tpe) tmp[t] = hw[t % nq] * fn_[t];
      csr_mul<double, NC>(nq, nq, op.D_ptr[m], op.D_idx[m], op.D_val[m], fn_, tmp2, lane, tpe);
      __syncthreads();
      // r_q += D_m^T tmp - halfWLambda .* tmp2
      for (int t = lane; t < NC * nq; t += tpe) {
        int i = t % nq, e = t / nq;
        double acc = 0.0;
        for (int q = op.Dt_ptr[m][i]; q < op.Dt_ptr[m][i + 1]; ++q)
          acc += op.Dt_val[m][q] * tmp[e * nq + op.Dt_idx[m][q]];
        rq[t] += acc;
        rq[t] -= tmp2[t] * hw[i];
      }
      __syncthreads();
    }
    // f_f -= halfN[n] .* (R f_n)
    for (int t = lane; t < NC * nf; t += tpe) {
      int j = t % nf, e = t / nf;
      double acc = 0.0;
      for (int q = op.R_ptr[j]; q < op.R_ptr[j + 1]; ++q) acc += op.R_val[q] * fn_[e * nq + op.R_idx[q]];
      double halfN = 0.5 * ka.geo.n_f[n + D * (j + (size_t)nf * kk)];
      ff[t] -= acc * halfN;
    }
    __syncthreads();
  }
  // f_f .*= BJf ; r_q -= R^T f_f
  for (int t = lane; t < NC * nf; t += tpe) ff[t] *= ka.geo.BJf[(size_t)kk * nf + t % nf];
  __syncthreads();
  rt_apply<double, NC>(op, op.Rt_val, ff, lane, tpe, [&](int t, double v) { rq[t] -= v; });
  __syncthreads();
  double *Xm = tmp, *Yq = tmp2;
  vdm_tmul<double, D, NC>(op, rq, Xm, Z, Wb, lane, tpe);
  mass_solve<double, D, NC>(op, ka.geo.JinvW ? ka.geo.JinvW + (size_t)kk * nq : nullptr,
                    ka.geo.WJinv ? ka.geo.WJinv + (size_t)kk * nq : nullptr, ka.mass_wa, Xm, Yq,
                    Z, Wb, lane, tpe, ka.Ak ? ka.Ak + (size_t)kk * op.np * op.np : nullptr);
  double *out = ka.dudt + (size_t)kk * NC * np;
  if (live)
    for (int t = lane; t < NC * np; t += tpe) {
      out[t] = Xm[t];
      if (!isfinite(Xm[t])) ka.flag_nonphysical();
    }
}

// ---------------------------------------------------------------------------
// Phase B of the mixed form, FluxDifferencingForm with the EC flux (Euler):
// the same steps as fd_time_derivative_kernel in FP32 on the perturbation
// states u_qf/u_ff written by phase A, FP32 metric terms and operators; the
// residual is written in FP64 for the FP64 stage accumulation.
//
// ET (a per-element tail operator E_k = A_k V^T [I | -R^T] exists): the
// volume and facet residuals live node-major in one array X (8 floats per
// node, volume nodes then facet nodes), and the lift R^T, V^T and the mass
// solve are one product with E_k, streamed from HBM (prefetched into L2 at
// entry) by all of the element's threads; otherwise r_q and f_f are
// component-major and the tail applies R^T, the sum-factorised V^T and the
// mass solve in turn.
// ---------------------------------------------------------------------------

// Node-major residuals of the tail product, in quads of four nodes: the
// first four components of node n are float4 (n & 3) of quad n >> 2, the
// fifth (NC = 5) is entry n & 3 of the quad's fifth float4, so that one
// column quad of E_k meets its 4 x NC values in four vector loads, plus one
// for the fifth components
template <int NC>
constexpr int kQuadFloats = NC > 4 ? 20 : 16;

template <int NC>
__device__ __forceinline__ int xq_index(int n, int e) {
  return (n >> 2) * kQuadFloats<NC> + (e < 4 ? (n & 3) * 4 + e : 16 + (n & 3));
}

template <int NC>
__device__ __forceinline__ void store_xq(float *X, int n, const float *v) {
  float *q = X + (n >> 2) * kQuadFloats<NC>;
  *reinterpret_cast<float4 *>(q + (n & 3) * 4) = make_float4(v[0], v[1], v[2], v[3]);
  if constexpr (NC > 4) q[16 + (n & 3)] = v[4];
}

template <int NC>
__device__ __forceinline__ void load_xq(const float *X, int n, float *v) {
  const float *q = X + (n >> 2) * kQuadFloats<NC>;
  const float4 a = *reinterpret_cast<const float4 *>(q + (n & 3) * 4);
  v[0] = a.x;
  v[1] = a.y;
  v[2] = a.z;
  v[3] = a.w;
  if constexpr (NC > 4) v[4] = q[16 + (n & 3)];
}

// x[n] -= v for node n
template <int NC>
__device__ __forceinline__ void sub_xq(float *X, int n, const float *v) {
  float *q = X + (n >> 2) * kQuadFloats<NC>;
  float4 *p = reinterpret_cast<float4 *>(q + (n & 3) * 4);
  float4 a = *p;
  a.x -= v[0];
  a.y -= v[1];
  a.z -= v[2];
  a.w -= v[3];
  *p = a;
  if constexpr (NC > 4) q[16 + (n & 3)] -= v[4];
}

// acc[e] += E[r, 4q + u] X[4q + u][e] for the four nodes of the column quad
// at Xq
template <int NC>
__device__ __forceinline__ void quad_fma(const float *Xq, float4 ev, float *acc) {
  const float w[4] = {ev.x, ev.y, ev.z, ev.w};
  float c4[4] = {0.f, 0.f, 0.f, 0.f};
  if constexpr (NC > 4) {
    const float4 t = *reinterpret_cast<const float4 *>(Xq + 16);
    c4[0] = t.x;
    c4[1] = t.y;
    c4[2] = t.z;
    c4[3] = t.w;
  }
#pragma unroll
  for (int u = 0; u < 4; ++u) {
    const float4 x0 = *reinterpret_cast<const float4 *>(Xq + 4 * u);
    acc[0] = fmaf(w[u], x0.x, acc[0]);
    acc[1] = fmaf(w[u], x0.y, acc[1]);
    acc[2] = fmaf(w[u], x0.z, acc[2]);
    acc[3] = fmaf(w[u], x0.w, acc[3]);
    if constexpr (NC > 4) acc[4] = fmaf(w[u], c4[u], acc[4]);
  }
}

// one node's NC values into an 8-float slot (the tail's partial rows)
template <int NC>
__device__ __forceinline__ void store_node(float *x, const float *v) {
  *reinterpret_cast<float4 *>(x) = make_float4(v[0], v[1], v[2], v[3]);
#pragma unroll
  for (int e = 4; e < NC; ++e) x[e] = v[e];
}

// Pair buffer of the mixed phase B: the first four components of pair p as
// float4 p of the buffer, the fifth (NC = 5) at 4 ch + p (ch pairs per chunk)
template <int NC>
__device__ __forceinline__ void store_pair(float *d, int ch, int p, const float *v) {
  reinterpret_cast<float4 *>(d)[p] = make_float4(v[0], v[1], v[2], v[3]);
  if constexpr (NC > 4) d[4 * ch + p] = v[4];
}

template <int NC>
__device__ __forceinline__ void load_pair(const float *d, int ch, int p, float *v) {
  const float4 a = reinterpret_cast<const float4 *>(d)[p];
  v[0] = a.x;
  v[1] = a.y;
  v[2] = a.z;
  v[3] = a.w;
  if constexpr (NC > 4) v[4] = d[4 * ch + p];
}

template <int D, int NC, bool ET>
__global__ void __launch_bounds__(256, 4) fd_time_derivative_mixed_kernel(KernelArgs ka) {
  static_assert(NC == D + 2, "the mixed form covers the Euler equations");
  static_assert(NC <= 5, "pair buffer and primitives hold at most five components");
  extern __shared__ __align__(16) double smem_raw[];
  float *smem = reinterpret_cast<float *>(smem_raw);
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const DevGeo &g = ka.geo;
  const Layout &L = ka.layBm;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq, nf = op.nf, nfac = op.nfac, npf = op.npf;
  const float rnpf = qrcp(npf > 0 ? npf : 1);
  float *base = smem + (size_t)team * L.team_doubles;  // team size in floats for this layout
  float *rq = base + L.off[0], *ff = base + L.off[2], *diff = base + L.off[4], *prim = base + L.off[7];
  float *X = base + L.off[2];  // ET: node-major residuals (region 2)
  // residual entries of volume node i / facet node j, component e
  auto RQ = [&](int e, int i) -> float & {
    if constexpr (ET) return X[xq_index<NC>(i, e)];
    else return rq[e * nq + i];
  };
  auto FF = [&](int e, int j) -> float & {
    if constexpr (ET) return X[xq_index<NC>(nq + j, e)];
    else return ff[e * nf + j];
  };
  const float *Ekg = ET ? ka.Ekf + (size_t)kk * ka.ek_quads * np * 4 : nullptr;
  if constexpr (ET) {
    if (lane == 0) prefetch_l2(Ekg, (uint32_t)ka.ek_quads * np * 16);
    // padding nodes of the last column quad: zero (E_k is zero there too)
    for (int t = lane; t < (4 * ka.ek_quads - nq - nf) * NC; t += tpe) X[xq_index<NC>(nq + nf + t / NC, t % NC)] = 0.f;
  }
  uint64_t *bar = reinterpret_cast<uint64_t *>(base + L.off[10]);
  constexpr int PS = 4 + D;
  const float gm1 = ph.f_gm1, igm1 = ph.f_igm1, gam = ph.f_gamma;
  const float rho_ref = ph.f_rho_ref, p_ref = ph.f_p_ref, hl = ph.f_half_lambda;
  const float theta_ref = ph.f_theta_ref, H_ref = ph.f_H_ref;

  // The element's slabs (FP32 nodal states, Lambda_q, halfnJq, and where
  // the layout gives them room the facet geometry, the mass operator and the
  // reference residual) move into shared memory as bulk copies issued by one
  // thread of the team, completed on the team's mbarrier.
  const float *uqg = ka.u_qf + (size_t)kk * NC * nq;
  const float *ufg = ka.u_ff + (size_t)kk * NC * nf;
  constexpr int LS = lambda_stride(D);
  const float *Lg = g.Lambda_qn + (size_t)kk * nq * LS;
  const float *Hg = g.halfnJqt + (size_t)kk * D * nfac * nq;
  const float *nfg = g.n_ff + (size_t)kk * D * nf, *bjg = g.BJff + (size_t)kk * nf;
  const float *hfg = g.halfnJff + (size_t)kk * D * nf;
  const float *Akg = ka.Akf ? ka.Akf + (size_t)kk * np * np : nullptr;
  const double *Rg = g.Rref ? g.Rref + (size_t)kk * NC * np : nullptr;
  const bool st_ak = Akg && L.off[4] > L.off[3];
  const bool st_geo = L.off[9] > L.off[8];
  const bool st_rref = Rg && L.off[10] > L.off[9];
  const bool st_hnq = op.nfp > 0;
  float *geo_r = base + L.off[8];
  float *geo_b = geo_r + ((D * nf + 8 + 3) & ~3), *geo_h = geo_b + ((nf + 8 + 3) & ~3);
  const float *uq = staged_ptr(base + L.off[0], uqg), *uf = staged_ptr(base + L.off[1], ufg);
  const float *Lam = staged_ptr(base + L.off[5], Lg);
  const float *hnq = staged_ptr(base + L.off[6], Hg);  // read only where there are facet pairs
  const float *nfv = st_geo ? staged_ptr(geo_r, nfg) : nfg, *bjf = st_geo ? staged_ptr(geo_b, bjg) : bjg;
  const float *hnf = st_geo ? staged_ptr(geo_h, hfg) : hfg;
  const float *Aks = st_ak ? staged_ptr(base + L.off[3], Akg) : Akg;
  const double *Rs = st_rref ? staged_ptr(base + L.off[9], Rg) : Rg;
  if (lane == 0) {
    mbar_init(bar, 1);
    mbar_fence_init();
    const uint32_t bq = NC * nq * 4, bf = NC * nf * 4, bl = nq * LS * 4, bh = D * nfac * nq * 4;
    const uint32_t bn = D * nf * 4, bb = nf * 4, ba = np * np * 4, br = NC * np * 8;
    uint32_t tx = staged_span(uqg, bq) + staged_span(ufg, bf) + staged_span(Lg, bl);
    if (st_hnq) tx += staged_span(Hg, bh);
    if (st_geo) tx += staged_span(nfg, bn) + staged_span(bjg, bb) + staged_span(hfg, bn);
    if (st_ak) tx += staged_span(Akg, ba);
    if (st_rref) tx += staged_span(Rg, br);
    mbar_arrive_expect_tx(bar, tx);
    stage_slab(base + L.off[0], uqg, bq, bar);
    stage_slab(base + L.off[1], ufg, bf, bar);
    stage_slab(base + L.off[5], Lg, bl, bar);
    if (st_hnq) stage_slab(base + L.off[6], Hg, bh, bar);
    if (st_geo) {
      stage_slab(geo_r, nfg, bn, bar);
      stage_slab(geo_b, bjg, bb, bar);
      stage_slab(geo_h, hfg, bn, bar);
    }
    if (st_ak) stage_slab(base + L.off[3], Akg, ba, bar);
    if (st_rref) stage_slab(base + L.off[9], Rg, br, bar);
  }
  // With all volume pairs in one chunk, the interface flux of facet node j
  // runs in the volume-sum phase, on the thread of node n_q + j of the node
  // loop (threads past the n_q volume nodes are idle there); else before
  // the pairs, on thread j.  Meanwhile: the neighbour's facet state of this
  // thread's first facet node (its gather overlaps the bulk copies), kept
  // in the node's residual slot (not staged, written by the interface flux
  // only) when the flux comes late.
  const bool iface_late = op.nvp > 0 && ka.fd_chunk_mixed >= op.nvp;
  const int j0 = iface_late ? lane + (lane >= nq ? 0 : (nq - lane + tpe - 1) / tpe) * tpe - nq : lane;
  float uo0[NC];
  if (j0 < nf) {
    const int P0 = __ldg(g.mapP + (size_t)kk * nf + j0);
    const int jn = P0 % nf, kn = P0 / nf;
#pragma unroll
    for (int e = 0; e < NC; ++e) uo0[e] = ka.u_ff[((size_t)kn * NC + e) * nf + jn];
    if (iface_late) {
      if constexpr (ET) store_xq<NC>(X, nq + j0, uo0);
      else
#pragma unroll
        for (int e = 0; e < NC; ++e) FF(e, j0) = uo0[e];
    }
  }
  __syncthreads();  // the mbarrier is initialised
  // one thread of the team waits for the copies; the others wait at the
  // barrier, where they take no issue slots (the barrier then orders the
  // landed data before their reads)
  const bool landed = lane != 0 ? true : mbar_wait_bounded(bar, 0);
  if (!__syncthreads_and(landed)) {
    if (lane == 0) ka.flag_timeout();
    mbar_wait_bounded(bar, 0);  // give copies still in flight a bounded time to land
    return;
  }
  for (int i = lane; i < nq + nf; i += tpe) {
    float du[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) du[e] = (i < nq) ? uq[e * nq + i] : uf[e * nf + (i - nq)];
    euler_prim_mixed<D>(gm1, rho_ref, p_ref, du, prim + (int)i * PS);
  }
  __syncthreads();

  // interface flux: EC flux . n + Lax-Friedrichs, scaled by BJf
  auto interface_flux = [&](int j, bool late) {
    float uo[NC], n[D], Po[4 + D], out[NC];
    if (j == j0) {
      if (late && ET) load_xq<NC>(X, nq + j, uo);
      else
#pragma unroll
        for (int e = 0; e < NC; ++e) uo[e] = late ? FF(e, j) : uo0[e];
    } else {
      const int P = g.mapP[(size_t)kk * nf + j];
      const int jn = P % nf, kn = P / nf;
#pragma unroll
      for (int e = 0; e < NC; ++e) uo[e] = ka.u_ff[((size_t)kn * NC + e) * nf + jn];
    }
#pragma unroll
    for (int m = 0; m < D; ++m) n[m] = nfv[m + D * j];
    const float *Pi = prim + (int)(nq + j) * PS;
    euler_prim_mixed<D>(gm1, rho_ref, p_ref, uo, Po);
    ec_flux_dot_mixed<D>(igm1, rho_ref, theta_ref, Pi, Po, n, out);
    float a = 0.f;
    if (ph.nflux == 0) {
      float vni = 0.f, vno = 0.f;
#pragma unroll
      for (int m = 0; m < D; ++m) { vni = fmaf(Pi[3 + m], n[m], vni); vno = fmaf(Po[3 + m], n[m], vno); }
      float ci = sqrtf(gam * (theta_ref + Pi[2])), co = sqrtf(gam * (theta_ref + Po[2]));
      a = hl * (fmaxf(fabsf(vni), fabsf(vno)) + fmaxf(ci, co));
    }
    const float bj = bjf[j];
    float jump[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) jump[e] = uf[e * nf + j] - uo[e];
    jump[NC - 1] = fmaf(-H_ref, jump[0], jump[NC - 1]);  // reduced energy: E' - H_ref rho'
    float res[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) res[e] = ((ph.nflux == 0) ? fmaf(a, jump[e], out[e]) : out[e]) * bj;
    if constexpr (ET) store_xq<NC>(X, nq + j, res);
    else
#pragma unroll
      for (int e = 0; e < NC; ++e) FF(e, j) = res[e];
  };
  if (!iface_late)
    for (int j = lane; j < nf; j += tpe) interface_flux(j, false);

  // volume flux differencing: one contracted EC flux per unique pair, in
  // chunks of at most CH pairs with per-node cursors (ascending pair order)
  const float4 *vpk = reinterpret_cast<const float4 *>(op.vp_pkf);
  const int CH = ka.fd_chunk_mixed;
  int cur[kMaxNodeSlots];
#pragma unroll
  for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
    const int i = lane + sl * tpe;
    cur[sl] = i < nq ? op.vp_inc_ptr[i] : 0;
    if (i < nq && CH < op.nvp)
      for (int e = 0; e < NC; ++e) RQ(e, i) = 0.f;
  }
  for (int c0 = 0; c0 < op.nvp; c0 += CH) {
    const int c1 = min(op.nvp, c0 + CH);
    float4 nx = c0 + lane < c1 ? __ldg(vpk + c0 + lane) : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int pidx = c0 + lane; pidx < c1; pidx += tpe) {
      const float4 cu = nx;
      if (pidx + tpe < c1) nx = __ldg(vpk + pidx + tpe);
      const int ij = __float_as_int(cu.w);
      const float Sv[3] = {cu.x, cu.y, cu.z};
      int i = ij & 0xffff, j = ij >> 16;
      float G[D], out[NC];
#pragma unroll
      for (int n = 0; n < D; ++n) G[n] = 0.f;
#pragma unroll
      for (int m = 0; m < D; ++m) {
        const float Sm = Sv[m];
        if (Sm == 0.f) continue;
#pragma unroll
        for (int n = 0; n < D; ++n) G[n] = fmaf(Sm, Lam[i * LS + m + D * n] + Lam[j * LS + m + D * n], G[n]);
      }
      ec_flux_dot_mixed<D>(igm1, rho_ref, theta_ref, prim + (int)i * PS, prim + (int)j * PS, G, out);
      store_pair<NC>(diff, CH, pidx - c0, out);
    }
    __syncthreads();
    if (CH >= op.nvp) {
      // one chunk: each node sums its whole incidence list; the threads of
      // the facet nodes compute the interface flux meanwhile
      for (int i = lane; i < nq + nf; i += tpe) {
        if (i >= nq) {
          interface_flux(i - nq, true);
          continue;
        }
        float acc[NC];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = 0.f;
        const int qa = op.vp_inc_ptr[i], qb = op.vp_inc_ptr[i + 1];
        int q = qa;
        for (; q + 4 <= qb; q += 4) {
          int inc[4];
#pragma unroll
          for (int r = 0; r < 4; ++r) inc[r] = __ldg(op.vp_inc + q + r);
#pragma unroll
          for (int r = 0; r < 4; ++r) {
            float dp[NC];
            load_pair<NC>(diff, CH, inc[r] >> 1, dp);
            const float sg = (inc[r] & 1) ? -1.f : 1.f;
#pragma unroll
            for (int e = 0; e < NC; ++e) acc[e] = fmaf(sg, dp[e], acc[e]);
          }
        }
        for (; q < qb; ++q) {
          const int inc = __ldg(op.vp_inc + q);
          float dp[NC];
          load_pair<NC>(diff, CH, inc >> 1, dp);
          const float sg = (inc & 1) ? -1.f : 1.f;
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] = fmaf(sg, dp[e], acc[e]);
        }
        if constexpr (ET) store_xq<NC>(X, i, acc);
        else
#pragma unroll
          for (int e = 0; e < NC; ++e) rq[e * nq + i] = acc[e];
      }
      __syncthreads();
      continue;
    }
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int i = lane + sl * tpe;
      if (i >= nq) continue;
      float acc[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) acc[e] = RQ(e, i);
      int q = cur[sl];
      const int qe = op.vp_inc_ptr[i + 1];
      for (; q < qe; ++q) {
        const int inc = op.vp_inc[q];
        const int pidx = inc >> 1;
        if (pidx >= c1) break;
        float dp[NC];
        load_pair<NC>(diff, CH, pidx - c0, dp);
        if (inc & 1) {
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] -= dp[e];
        } else {
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] += dp[e];
        }
      }
      cur[sl] = q;
#pragma unroll
      for (int e = 0; e < NC; ++e) RQ(e, i) = acc[e];
    }
    __syncthreads();
  }

  // facet correction, chunked the same way
  if (op.nfp > 0) {
    const float2 *fpk = reinterpret_cast<const float2 *>(op.fp_pkf);
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int t = lane + sl * tpe;
      cur[sl] = t < nq ? op.fp_q_ptr[t] : (t < nq + nf ? op.fp_f_ptr[t - nq] : 0);
    }
    for (int c0 = 0; c0 < op.nfp; c0 += CH) {
      const int c1 = min(op.nfp, c0 + CH);
      float2 nx = c0 + lane < c1 ? __ldg(fpk + c0 + lane) : make_float2(0.f, 0.f);
      for (int pidx = c0 + lane; pidx < c1; pidx += tpe) {
        const float2 cu = nx;
        if (pidx + tpe < c1) nx = __ldg(fpk + pidx + tpe);
        const int ij = __float_as_int(cu.y);
        const float Cij = cu.x;
        int i = ij & 0xffff, j = ij >> 16;
        int f = qdiv(j, rnpf);
        float G[D], out[NC];
#pragma unroll
        for (int m = 0; m < D; ++m) G[m] = Cij * (hnf[m + D * j] + hnq[(f * D + m) * nq + i]);
        ec_flux_dot_mixed<D>(igm1, rho_ref, theta_ref, prim + (int)i * PS, prim + (int)(nq + j) * PS, G, out);
        store_pair<NC>(diff, CH, pidx - c0, out);
      }
      __syncthreads();
      if (CH >= op.nfp) {
        // one chunk: each node sums its whole incidence list
        for (int t = lane; t < nq + nf; t += tpe) {
          float acc[NC];
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] = 0.f;
          const bool vol = t < nq;
          const int r = vol ? t : t - nq;
          const int *ptr = vol ? op.fp_q_ptr : op.fp_f_ptr;
          const int qa = ptr[r], qb = ptr[r + 1];
          if (vol) {
            int q = qa;
            for (; q + 4 <= qb; q += 4) {
              int id[4];
#pragma unroll
              for (int u = 0; u < 4; ++u) id[u] = __ldg(op.fp_q + q + u);
#pragma unroll
              for (int u = 0; u < 4; ++u) {
                float dp[NC];
                load_pair<NC>(diff, CH, id[u], dp);
#pragma unroll
                for (int e = 0; e < NC; ++e) acc[e] += dp[e];
              }
            }
            for (; q < qb; ++q) {
              float dp[NC];
              load_pair<NC>(diff, CH, __ldg(op.fp_q + q), dp);
#pragma unroll
              for (int e = 0; e < NC; ++e) acc[e] += dp[e];
            }
          } else {
            // the pairs are enumerated facet node by facet node (the columns
            // of C): a facet node's pairs are the consecutive ids qa..qb-1
            for (int q = qa; q < qb; ++q) {
              float dp[NC];
              load_pair<NC>(diff, CH, q, dp);
#pragma unroll
              for (int e = 0; e < NC; ++e) acc[e] += dp[e];
            }
          }
          if constexpr (ET) {
            sub_xq<NC>(X, t, acc);
          } else {
            float *dst = vol ? rq + r : ff + r;
            const int stride = vol ? nq : nf;
#pragma unroll
            for (int e = 0; e < NC; ++e) dst[e * stride] -= acc[e];
          }
        }
        __syncthreads();
        continue;
      }
#pragma unroll
      for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
        const int t = lane + sl * tpe;
        if (t >= nq + nf) continue;
        float acc[NC];
#pragma unroll
        for (int e = 0; e < NC; ++e) acc[e] = 0.f;
        const bool vol = t < nq;
        const int r = vol ? t : t - nq;
        const int qe = vol ? op.fp_q_ptr[r + 1] : op.fp_f_ptr[r + 1];
        int q = cur[sl];
        for (; q < qe; ++q) {
          // a facet node's pairs are its consecutive ids (C's columns)
          const int pidx = vol ? __ldg(op.fp_q + q) : q;
          if (pidx >= c1) break;
          float dp[NC];
          load_pair<NC>(diff, CH, pidx - c0, dp);
#pragma unroll
          for (int e = 0; e < NC; ++e) acc[e] += dp[e];
        }
        cur[sl] = q;
        if constexpr (ET) {
          sub_xq<NC>(X, t, acc);
        } else {
          float *dst = vol ? rq + r : ff + r;
          const int stride = vol ? nq : nf;
#pragma unroll
          for (int e = 0; e < NC; ++e) dst[e * stride] -= acc[e];
        }
      }
      __syncthreads();
    }
  }

  // energy residual = H_ref x density residual + reduced-flux residual, in
  // FP64, plus the reference state's own FP64 residual (the dropped
  // reference-pressure terms)
  double *outp = ka.dudt + (size_t)kk * NC * np;
  const double *rref = Rs;
  if constexpr (ET) {
    // out = E_k [r_q ; f_f]: thread (g, r) sums the column quads g, g + G,
    // ... of row r (four loads in flight in 3-D, three in 2-D); the G
    // partial rows are added in a fixed order by the row's thread
    const int G = tpe / np, gq = lane / np, r = lane - gq * np;
    const int nquad = ka.ek_quads;
    const float4 *E4 = reinterpret_cast<const float4 *>(Ekg);
    float acc[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) acc[e] = 0.f;
    if (gq < G) {
      int q = gq;
      if constexpr (D == 3) {
        // four loads in flight (p = 4 tets: 8 or 9 column quads per thread,
        // two rounds instead of four or five; 2 % faster, the 2-D kernel
        // spills with four)
        for (; q + 3 * G < nquad; q += 4 * G) {
          const float4 ea = __ldg(E4 + (size_t)q * np + r);
          const float4 eb = __ldg(E4 + (size_t)(q + G) * np + r);
          const float4 ec = __ldg(E4 + (size_t)(q + 2 * G) * np + r);
          const float4 ed = __ldg(E4 + (size_t)(q + 3 * G) * np + r);
          quad_fma<NC>(X + q * kQuadFloats<NC>, ea, acc);
          quad_fma<NC>(X + (q + G) * kQuadFloats<NC>, eb, acc);
          quad_fma<NC>(X + (q + 2 * G) * kQuadFloats<NC>, ec, acc);
          quad_fma<NC>(X + (q + 3 * G) * kQuadFloats<NC>, ed, acc);
        }
      } else {
        for (; q + 2 * G < nquad; q += 3 * G) {
          const float4 ea = __ldg(E4 + (size_t)q * np + r);
          const float4 eb = __ldg(E4 + (size_t)(q + G) * np + r);
          const float4 ec = __ldg(E4 + (size_t)(q + 2 * G) * np + r);
          quad_fma<NC>(X + q * kQuadFloats<NC>, ea, acc);
          quad_fma<NC>(X + (q + G) * kQuadFloats<NC>, eb, acc);
          quad_fma<NC>(X + (q + 2 * G) * kQuadFloats<NC>, ec, acc);
        }
      }
      for (; q < nquad; q += G) quad_fma<NC>(X + q * kQuadFloats<NC>, __ldg(E4 + (size_t)q * np + r), acc);
      store_node<NC>(diff + (gq * np + r) * 8, acc);
    }
    __syncthreads();
    if (live && lane < np) {
      float s[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) s[e] = 0.f;
      for (int gg = 0; gg < G; ++gg) {
        const float *pr = diff + (gg * np + lane) * 8;
#pragma unroll
        for (int e = 0; e < NC; ++e) s[e] += pr[e];
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        double v = (double)s[e];
        if (e == NC - 1) v = fma(ph.H_ref, (double)s[0], v);
        if (rref) v += rref[e * np + lane];
        outp[e * np + lane] = v;
        if (!isfinite(s[e])) ka.flag_nonphysical();
      }
    }
    return;
  }
  // r_q -= R^T f_f
  const float *Rt = OpVals<float>::Rt(op);
  rt_apply<float, NC>(op, Rt, ff, lane, tpe, [&](int t, float v) { rq[t] -= v; });
  __syncthreads();

  // the pair buffer holds the modal / nodal buffers and the scratch now
  float *Xm = diff, *Yq = diff + (int)NC * np;
  float *Z = Yq + (size_t)NC * nq;
  float *Wb = Z + ka.vdm_zsz_mixed;
  vdm_tmul<float, D, NC>(op, rq, Xm, Z, Wb, lane, tpe);
  mass_solve<float, D, NC>(op, g.JinvWf ? g.JinvWf + (size_t)kk * nq : nullptr,
                           g.WJinvf ? g.WJinvf + (size_t)kk * nq : nullptr, ka.mass_wa, Xm, Yq, Z,
                           Wb, lane, tpe, Aks);
  if (live)
    for (int t = lane; t < NC * np; t += tpe) {
      double v = (double)Xm[t];
      if (t >= (NC - 1) * np) v = fma(ph.H_ref, (double)Xm[t - (NC - 1) * np], v);
      if (rref) v += rref[t];
      outp[t] = v;
      if (!isfinite(Xm[t])) ka.flag_nonphysical();
    }
}

// ---------------------------------------------------------------------------
// element-wise helpers: time-integration updates, layout conversion, reductions
// ---------------------------------------------------------------------------

// CarpenterKennedy2N54 stage: tmp = a tmp + dt k ; u = u + b tmp (a = 0 on stage 1)
__global__ void ck_stage_kernel(double *__restrict__ u, double *__restrict__ tmp,
                                const double *__restrict__ k, double a, double b, double dt,
                                int first, size_t n) {
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
    double t = first ? dt * k[x] : a * tmp[x] + dt * k[x];
    tmp[x] = t;
    u[x] = u[x] + b * t;
  }
}

// The same stage with the update u += b tmp accumulated by compensated
// (Kahan) summation: comp carries the low-order part lost when the small
// increment is added to the state.  Used by the mixed form.
__global__ void ck_stage_compensated_kernel(double *__restrict__ u, double *__restrict__ comp,
                                            double *__restrict__ tmp, const double *__restrict__ k,
                                            double a, double b, double dt, int first, size_t n) {
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
    double t = first ? dt * k[x] : a * tmp[x] + dt * k[x];
    tmp[x] = t;
    double y = b * t - comp[x];
    double s = u[x] + y;
    comp[x] = (s - u[x]) - y;
    u[x] = s;
  }
}

// FP64 -> FP32 rounding of metric terms and operator values for the mixed form
// Every volume and facet node of every element set to one constant state
// (FP64 nodal scratch layouts: u_q element-major (nq, nc) blocks, u_f
// element-major (nf, nc) blocks): the nodal states of the mixed form's
// reference state, whose phase-B residual the mixed form adds back.
__global__ void fill_constant_state_kernel(double *__restrict__ buf, int nodes, int nc, size_t n,
                                           double s0, double s1, double s2, double s3, double s4) {
  const double s[5] = {s0, s1, s2, s3, s4};
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    buf[i] = s[(i / nodes) % nc];
}

// out = (float)(in + shift)
__global__ void round_to_float_kernel(const double *__restrict__ in, float *__restrict__ out, size_t n,
                                      double shift) {
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x)
    out[x] = (float)(in[x] + shift);
}

// FP64 -> FP32 rounding of Lambda_q (v n_q + i per element) into the
// node-major layout lambda_stride(d) i + v (padding entries zero)
__global__ void lambda_node_major_kernel(const double *__restrict__ in, float *__restrict__ out, size_t ne,
                                         int nq, int d) {
  const int ls = lambda_stride(d), dd = d * d, per = nq * ls;
  const size_t n = ne * (size_t)per;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
    const size_t k = x / per;
    const int t = (int)(x - k * per);
    const int i = t / ls, v = t - i * ls;
    out[x] = v < dd ? (float)in[k * (size_t)nq * dd + (size_t)v * nq + i] : 0.f;
  }
}

// The mixed phase B's packed pair tables (FP32 roundings of S and C with
// the packed node indices' bits)
__global__ void pack_pairs_kernel(const int *__restrict__ vp_ij, const double *__restrict__ vp_S, int nvp,
                                  const int *__restrict__ fp_ij, const double *__restrict__ fp_C, int nfp, int d,
                                  float4 *__restrict__ vpk, float2 *__restrict__ fpk) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nvp + nfp; t += gridDim.x * blockDim.x) {
    if (t < nvp) {
      float s[3] = {0.f, 0.f, 0.f};
      for (int m = 0; m < d; ++m) s[m] = (float)vp_S[(size_t)t * d + m];
      vpk[t] = make_float4(s[0], s[1], s[2], __int_as_float(vp_ij[t]));
    } else {
      const int q = t - nvp;
      fpk[q] = make_float2((float)fp_C[q], __int_as_float(fp_ij[q]));
    }
  }
}

// FP64 -> FP32 rounding of halfnJq (m + D (f + nfac i) per element) into the
// layout (f D + m) n_q + i; one thread per output float
__global__ void halfnjq_transpose_kernel(const double *__restrict__ in, float *__restrict__ out, size_t ne,
                                         int nq, int d, int nfac) {
  const int per = d * nfac * nq;
  const size_t n = ne * (size_t)per;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
    const size_t k = x / per;
    const int t = (int)(x - k * per);
    const int fm = t / nq, i = t - fm * nq;
    const int f = fm / d, m = fm - f * d;
    out[x] = (float)in[k * per + m + d * (f + nfac * i)];
  }
}

// FP64 -> FP32 rounding of nmat n x n matrices with a transpose of each: the
// column-major FP64 mass operators become row-major FP32 ones
__global__ void round_transpose_kernel(const double *__restrict__ in, float *__restrict__ out, size_t nmat,
                                       int n) {
  const size_t nn = (size_t)n * n, total = nmat * nn;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < total; x += (size_t)gridDim.x * blockDim.x) {
    const size_t k = x / nn;
    const int r = (int)(x - k * nn), a = r / n, b = r - a * n;
    out[x] = (float)in[k * nn + (size_t)b * n + a];
  }
}

// classic RK4 stage helpers
__global__ void rk4_stage_kernel(const double *__restrict__ u, double *__restrict__ ust,
                                 double *__restrict__ acc, const double *__restrict__ k,
                                 double acc_w, double c, int first, size_t n) {
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
    double kx = k[x];
    acc[x] = first ? kx : acc[x] + acc_w * kx;
    ust[x] = u[x] + c * kx;
  }
}

__global__ void rk4_final_kernel(double *__restrict__ u, const double *__restrict__ acc,
                                 const double *__restrict__ k, double dt6, size_t n) {
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x)
    u[x] = u[x] + dt6 * (acc[x] + k[x]);
}

// internal facet layout (ne, nc, nf) -> the reference's (nf, ne, nc)
__global__ void facet_to_reference_layout(const double *__restrict__ in, double *__restrict__ out,
                                          int nf, int ne, int nc) {
  size_t n = (size_t)nf * ne * nc;
  for (size_t x = blockIdx.x * (size_t)blockDim.x + threadIdx.x; x < n; x += (size_t)gridDim.x * blockDim.x) {
    size_t j = x % nf, r = x / nf, k = r % ne, e = r / ne;
    out[x] = in[(k * nc + e) * nf + j];
  }
}

// per-element FP64 partial sums of the conservation and entropy residuals
// (Analysis/conservation.jl:145-189); reduced on the host in element order
template <int D, int NC>
__global__ void __launch_bounds__(256) conservation_kernel(KernelArgs ka, const double *u,
                                                           const double *dudt, double *partial) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Layout &L = ka.layA;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  double *base = smem + (size_t)team * L.team_doubles;
  double *X = base + L.off[0], *Y = base + L.off[1], *Z = base + L.off[2], *Wb = base + L.off[3],
         *F = base + L.off[4];
  const int np = op.np, nq = op.nq;
  for (int t = lane; t < NC * np; t += tpe) X[t] = u[(size_t)kk * NC * np + t];
  __syncthreads();
  vdm_mul<double, D, NC>(op, X, Y, Z, Wb, lane, tpe);       // Y = V u
  for (int t = lane; t < NC * np; t += tpe) X[t] = dudt[(size_t)kk * NC * np + t];
  __syncthreads();
  vdm_mul<double, D, NC>(op, X, F, Z, Wb, lane, tpe);       // F = V dudt
  const double *WJ = ka.geo.WJ + (size_t)kk * nq;
  // lane-ordered partial sums, reduced by lane 0 in a fixed order
  double *red = base + L.off[5];  // tpe x (NC + 1)
  {
    double acc[NC + 1];
#pragma unroll
    for (int e = 0; e <= NC; ++e) acc[e] = 0.0;
    for (int i = lane; i < nq; i += tpe) {
      double ui[NC], wi[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) ui[e] = Y[e * nq + i];
      if constexpr (NC > 1) cons_to_entropy<D>(ka.ph, ui, wi);
      else wi[0] = ui[0];
      double t = 0.0;
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        acc[e] += WJ[i] * F[e * nq + i];
        t += wi[e] * F[e * nq + i];
      }
      acc[NC] += WJ[i] * t;
    }
#pragma unroll
    for (int e = 0; e <= NC; ++e) red[lane * (NC + 1) + e] = acc[e];
  }
  __syncthreads();
  if (lane == 0 && live) {
    for (int e = 0; e <= NC; ++e) {
      double s = 0.0;
      for (int l = 0; l < tpe; ++l) s += red[l * (NC + 1) + e];
      partial[(size_t)k * (NC + 1) + e] = s;
    }
  }
}

// The weight-adjusted mass operator V' diag(J^-1 W) V of every element
// (mass_matrix.jl:185-196 applies it as V' (J^-1 W .* (V x))), built once
// column by column from the sum-factorised operator applied to unit
// vectors, n_p x n_p column-major per element.
template <int D, int NC>
__global__ void __launch_bounds__(256) mass_operator_kernel(KernelArgs ka, double *Ak) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Layout &L = ka.layA;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq;
  double *base = smem + (size_t)team * L.team_doubles;
  double *X = base + L.off[0], *Y = base + L.off[1], *Z = base + L.off[2], *Wb = base + L.off[3];
  const double *JinvW = ka.geo.JinvW + (size_t)kk * nq;
  double *out = Ak + (size_t)kk * np * np;
  for (int b0 = 0; b0 < np; b0 += NC) {
    for (int t = lane; t < NC * np; t += tpe) {
      const int e = t / np, l = t - e * np;
      X[t] = (l == b0 + e) ? 1.0 : 0.0;
    }
    __syncthreads();
    mass_solve<double, D, NC>(op, JinvW, nullptr, 1, X, Y, Z, Wb, lane, tpe);
    if (live)
      for (int t = lane; t < NC * np; t += tpe) {
        const int e = t / np, l = t - e * np;
        if (b0 + e < np) out[(size_t)(b0 + e) * np + l] = X[t];   // column b0 + e
      }
    __syncthreads();
  }
}

// EnergyConservationAnalysis (Analysis/conservation.jl:161-175):
// partial[k][e] = u[:, e, k]' M_k dudt[:, e, k] with the mass solver's mass
// matrix (mass_matrix.jl:150-158): WeightAdjustedSolver inv(V' diag(J^-1 W) V)
// (applied by a Cholesky solve of V' diag(J^-1 W) V, whose columns are the
// weight-adjusted operator applied to unit vectors), DiagonalSolver W J.
template <int D, int NC>
__global__ void __launch_bounds__(256) energy_kernel(KernelArgs ka, const double *u, const double *dudt,
                                                     double *partial) {
  extern __shared__ double smem[];
  __shared__ int bad;
  const DevOps &op = ka.op;
  const Layout &L = ka.layE;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq;
  double *base = smem + (size_t)team * L.team_doubles;
  double *X = base + L.off[0], *Y = base + L.off[1], *Z = base + L.off[2], *Wb = base + L.off[3],
         *A = base + L.off[4], *R = base + L.off[5];
  if (threadIdx.x == 0) bad = 0;
  for (int t = lane; t < NC * np; t += tpe) R[t] = dudt[(size_t)kk * NC * np + t];
  __syncthreads();
  if (ka.mass_wa) {
    const double *JinvW = ka.geo.JinvW + (size_t)kk * nq;
    // columns b0 .. b0 + NC - 1 of A = V' diag(J^-1 W) V per pass
    for (int b0 = 0; b0 < np; b0 += NC) {
      for (int t = lane; t < NC * np; t += tpe) {
        const int e = t / np, l = t - e * np;
        X[t] = (l == b0 + e) ? 1.0 : 0.0;
      }
      __syncthreads();
      mass_solve<double, D, NC>(op, JinvW, nullptr, 1, X, Y, Z, Wb, lane, tpe);
      for (int t = lane; t < NC * np; t += tpe) {
        const int e = t / np, l = t - e * np;
        if (b0 + e < np) A[l * np + (b0 + e)] = X[t];
      }
      __syncthreads();
    }
    team_cholesky_solve(A, np, R, NC, lane, tpe, &bad);  // R <- A^-1 dudt = M_WA dudt
  } else {
    const double *WJ = ka.geo.WJ + (size_t)kk * nq;  // n_p == n_q: M = diag(W J)
    for (int t = lane; t < NC * np; t += tpe) R[t] *= WJ[t % np];
    __syncthreads();
  }
  if (lane < NC && live) {
    const double *uk = u + (size_t)kk * NC * np + (size_t)lane * np;
    double s = 0.0;
    for (int l = 0; l < np; ++l) s = fma(uk[l], R[lane * np + l], s);
    partial[(size_t)k * NC + lane] = s;
  }
  if (threadIdx.x == 0 && bad) ka.flag_nonphysical();
}

// ---------------------------------------------------------------------------
// launch wrappers
// ---------------------------------------------------------------------------
#define SSE_DISPATCH(D_, NC_, CALL)                                       \
  if (ka.op.d == 2 && ka.op.nc == 1) { constexpr int D = 2, NC = 1; CALL; } \
  else if (ka.op.d == 2 && ka.op.nc == 4) { constexpr int D = 2, NC = 4; CALL; } \
  else if (ka.op.d == 3 && ka.op.nc == 1) { constexpr int D = 3, NC = 1; CALL; } \
  else if (ka.op.d == 3 && ka.op.nc == 5) { constexpr int D = 3, NC = 5; CALL; } \
  else return cudaErrorInvalidValue;

cudaError_t sse_set_smem_limits(const KernelArgs &ka, size_t smA, size_t smB) {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void *f, size_t bytes) {
    if (e == cudaSuccess) e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  };
  SSE_DISPATCH(D, NC, {
    set((const void *)nodal_values_kernel<D, NC>, smA);
    set((const void *)conservation_kernel<D, NC>, smA);
    if (ka.fd) set((const void *)fd_time_derivative_kernel<D, NC>, smB);
    else set((const void *)std_time_derivative_kernel<D, NC>, smB);
  });
  return e;
}

cudaError_t launch_nodal_values(const KernelArgs &ka, cudaStream_t st) {
  int grid = (ka.ne + ka.epb - 1) / ka.epb;
  if (ka.mixed && ka.op.has_vdm && ka.geo.P1) {
    // the mixed phase A has its own team geometry (epb_am elements per block
    // of the same tpb threads)
    KernelArgs km = ka;
    km.epb = ka.epb_am;
    const int grida = (ka.ne + km.epb - 1) / km.epb;
    size_t sm = (size_t)km.epb * ka.layAm.team_doubles * sizeof(double);
    if (ka.op.d == 2 && ka.op.nc == 4) nodal_values_mixed_kernel<2, 4><<<grida, ka.tpb, sm, st>>>(km);
    else if (ka.op.d == 3 && ka.op.nc == 5) nodal_values_mixed_kernel<3, 5><<<grida, ka.tpb, sm, st>>>(km);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
  }
  // the FP64 phase A has its own team geometry (epb_a elements per block of
  // the same tpb threads)
  KernelArgs ka2 = ka;
  ka2.epb = ka.epb_a;
  const int grid2 = (ka.ne + ka2.epb - 1) / ka2.epb;
  size_t sm = (size_t)ka2.epb * ka.layA.team_doubles * sizeof(double);
  SSE_DISPATCH(D, NC, (nodal_values_kernel<D, NC><<<grid2, ka.tpb, sm, st>>>(ka2)));
  return cudaGetLastError();
}

cudaError_t launch_projection_of_one(const KernelArgs &ka, double *P1, double *RP1, cudaStream_t st) {
  int grid = (ka.ne + ka.epb - 1) / ka.epb;
  size_t sm = (size_t)ka.epb * ka.layP1.team_doubles * sizeof(double);
  if (ka.op.d == 2) projection_of_one_kernel<2><<<grid, ka.tpb, sm, st>>>(ka, P1, RP1);
  else projection_of_one_kernel<3><<<grid, ka.tpb, sm, st>>>(ka, P1, RP1);
  return cudaGetLastError();
}

cudaError_t sse_set_smem_limits_mixed_a(const KernelArgs &ka) {
  cudaError_t e = cudaSuccess;
  const int am = (int)((size_t)ka.epb_am * ka.layAm.team_doubles * sizeof(double));
  const int p1 = (int)((size_t)ka.epb * ka.layP1.team_doubles * sizeof(double));
  if (ka.op.d == 2 && ka.op.nc == 4) {
    e = cudaFuncSetAttribute((const void *)nodal_values_mixed_kernel<2, 4>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, am);
  } else if (ka.op.d == 3 && ka.op.nc == 5) {
    e = cudaFuncSetAttribute((const void *)nodal_values_mixed_kernel<3, 5>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, am);
  } else {
    return cudaErrorInvalidValue;
  }
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(ka.op.d == 2 ? (const void *)projection_of_one_kernel<2>
                                          : (const void *)projection_of_one_kernel<3>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, p1);
  return e;
}

// the mixed phase-B instantiation of this configuration (with the tail
// operator where ka.Ekf is set), or null
static const void *mixed_b_kernel(const KernelArgs &ka) {
  const bool et = ka.Ekf != nullptr;
  if (ka.op.d == 2 && ka.op.nc == 4)
    return et ? (const void *)fd_time_derivative_mixed_kernel<2, 4, true>
              : (const void *)fd_time_derivative_mixed_kernel<2, 4, false>;
  if (ka.op.d == 3 && ka.op.nc == 5)
    return et ? (const void *)fd_time_derivative_mixed_kernel<3, 5, true>
              : (const void *)fd_time_derivative_mixed_kernel<3, 5, false>;
  return nullptr;
}

cudaError_t sse_mixed_b_blocks_per_sm(const KernelArgs &ka, size_t smBm, int *blocks) {
  const void *f = mixed_b_kernel(ka);
  if (!f) return cudaErrorInvalidValue;
  cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, 220 * 1024);
  if (e != cudaSuccess) return e;
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks, f, ka.tpb, smBm);
}

cudaError_t sse_set_smem_limit_mixed(const KernelArgs &ka, size_t smBm) {
  const void *f = mixed_b_kernel(ka);
  if (!f) return cudaErrorInvalidValue;
  return cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smBm);
}

cudaError_t launch_time_derivative(const KernelArgs &ka, cudaStream_t st) {
  int grid = (ka.ne + ka.epb - 1) / ka.epb;
  size_t sm = (size_t)ka.epb * ka.layB.team_doubles * sizeof(double);
  if (ka.mixed) {
    // the FP32 phase B has its own team geometry (epb_bm elements per block
    // of the same tpb threads)
    KernelArgs km = ka;
    km.epb = ka.epb_bm;
    const int gridm = (ka.ne + km.epb - 1) / km.epb;
    size_t smm = (size_t)km.epb * ka.layBm.team_doubles * sizeof(float);
    const bool et = ka.Ekf != nullptr;
    if (ka.op.d == 2 && ka.op.nc == 4) {
      if (et) fd_time_derivative_mixed_kernel<2, 4, true><<<gridm, ka.tpb, smm, st>>>(km);
      else fd_time_derivative_mixed_kernel<2, 4, false><<<gridm, ka.tpb, smm, st>>>(km);
    } else if (ka.op.d == 3 && ka.op.nc == 5) {
      if (et) fd_time_derivative_mixed_kernel<3, 5, true><<<gridm, ka.tpb, smm, st>>>(km);
      else fd_time_derivative_mixed_kernel<3, 5, false><<<gridm, ka.tpb, smm, st>>>(km);
    } else {
      return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
  if (ka.fd) {
    SSE_DISPATCH(D, NC, (fd_time_derivative_kernel<D, NC><<<grid, ka.tpb, sm, st>>>(ka)));
  } else {
    SSE_DISPATCH(D, NC, (std_time_derivative_kernel<D, NC><<<grid, ka.tpb, sm, st>>>(ka)));
  }
  return cudaGetLastError();
}

cudaError_t launch_mass_operator(const KernelArgs &ka, double *Ak, cudaStream_t st) {
  int grid = (ka.ne + ka.epb - 1) / ka.epb;
  size_t sm = (size_t)ka.epb * ka.layA.team_doubles * sizeof(double);
  cudaError_t e = cudaSuccess;
  SSE_DISPATCH(D, NC, (e = cudaFuncSetAttribute(mass_operator_kernel<D, NC>,
                                              cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)));
  if (e != cudaSuccess) return e;
  SSE_DISPATCH(D, NC, (mass_operator_kernel<D, NC><<<grid, ka.tpb, sm, st>>>(ka, Ak)));
  return cudaGetLastError();
}

cudaError_t launch_energy(const KernelArgs &ka, const double *u, const double *dudt, double *partial,
                          cudaStream_t st) {
  int grid = (ka.ne + ka.epb - 1) / ka.epb;
  size_t sm = (size_t)ka.epb * ka.layE.team_doubles * sizeof(double);
  cudaError_t e = cudaSuccess;
  SSE_DISPATCH(D, NC, (e = cudaFuncSetAttribute(energy_kernel<D, NC>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                              (int)sm)));
  if (e != cudaSuccess) return e;
  SSE_DISPATCH(D, NC, (energy_kernel<D, NC><<<grid, ka.tpb, sm, st>>>(ka, u, dudt, partial)));
  return cudaGetLastError();
}

cudaError_t launch_conservation(const KernelArgs &ka, const double *u, const double *dudt,
                                double *partial, cudaStream_t st) {
  int grid = (ka.ne + ka.epb - 1) / ka.epb;
  size_t sm = (size_t)ka.epb * ka.layA.team_doubles * sizeof(double);
  SSE_DISPATCH(D, NC, (conservation_kernel<D, NC><<<grid, ka.tpb, sm, st>>>(ka, u, dudt, partial)));
  return cudaGetLastError();
}

static int elementwise_grid(size_t n) {
  size_t g = (n + 255) / 256;
  return (int)(g > 152 * 16 ? 152 * 16 : (g < 1 ? 1 : g));
}

cudaError_t launch_ck_stage(double *u, double *tmp, const double *k, double a, double b, double dt,
                            int first, size_t n, cudaStream_t st) {
  ck_stage_kernel<<<elementwise_grid(n), 256, 0, st>>>(u, tmp, k, a, b, dt, first, n);
  return cudaGetLastError();
}

cudaError_t launch_ck_stage_compensated(double *u, double *comp, double *tmp, const double *k,
                                        double a, double b, double dt, int first, size_t n,
                                        cudaStream_t st) {
  ck_stage_compensated_kernel<<<elementwise_grid(n), 256, 0, st>>>(u, comp, tmp, k, a, b, dt, first, n);
  return cudaGetLastError();
}

cudaError_t launch_lambda_node_major(const double *in, float *out, size_t ne, int nq, int d, cudaStream_t st) {
  const size_t n = ne * (size_t)nq * lambda_stride(d);
  if (n == 0) return cudaSuccess;
  lambda_node_major_kernel<<<elementwise_grid(n), 256, 0, st>>>(in, out, ne, nq, d);
  return cudaGetLastError();
}

cudaError_t launch_pack_pairs(const DevOps &op, float *vpk, float *fpk, cudaStream_t st) {
  const int n = op.nvp + op.nfp;
  if (n == 0) return cudaSuccess;
  pack_pairs_kernel<<<(n + 255) / 256, 256, 0, st>>>(op.vp_ij, op.vp_S, op.nvp, op.fp_ij, op.fp_C, op.nfp, op.d,
                                                     reinterpret_cast<float4 *>(vpk),
                                                     reinterpret_cast<float2 *>(fpk));
  return cudaGetLastError();
}

cudaError_t launch_halfnjq_transpose(const double *in, float *out, size_t ne, int nq, int d, int nfac,
                                     cudaStream_t st) {
  const size_t n = ne * (size_t)d * nfac * nq;
  if (n == 0) return cudaSuccess;
  halfnjq_transpose_kernel<<<elementwise_grid(n), 256, 0, st>>>(in, out, ne, nq, d, nfac);
  return cudaGetLastError();
}

cudaError_t launch_round_to_float(const double *in, float *out, size_t n, cudaStream_t st, double shift) {
  if (n == 0) return cudaSuccess;
  round_to_float_kernel<<<elementwise_grid(n), 256, 0, st>>>(in, out, n, shift);
  return cudaGetLastError();
}

cudaError_t launch_fill_constant_state(double *buf, int nodes, int nc, size_t ne, const double *state,
                                       cudaStream_t st) {
  const size_t n = (size_t)nodes * nc * ne;
  if (n == 0) return cudaSuccess;
  double s[5] = {0, 0, 0, 0, 0};
  for (int e = 0; e < nc && e < 5; ++e) s[e] = state[e];
  fill_constant_state_kernel<<<elementwise_grid(n), 256, 0, st>>>(buf, nodes, nc, n, s[0], s[1], s[2], s[3], s[4]);
  return cudaGetLastError();
}

cudaError_t launch_round_transpose(const double *in, float *out, size_t nmat, int n, cudaStream_t st) {
  if (nmat == 0 || n == 0) return cudaSuccess;
  round_transpose_kernel<<<elementwise_grid(nmat * n * n), 256, 0, st>>>(in, out, nmat, n);
  return cudaGetLastError();
}

// Columns of M = V^T [I | -R^T] (n_p rows; column c at M + c n_p): V^T e_c
// for a volume node c, -(R V)^T e_j for facet node j = c - n_q, zero for the
// padding columns up to ncol.  Vd: dense V (n_q x n_p, column-major).
__global__ void tail_matrix_kernel(DevOps op, const double *__restrict__ Vd, double *__restrict__ M, int ncol) {
  const int np = op.np, nq = op.nq, nf = op.nf;
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < np * ncol; t += gridDim.x * blockDim.x) {
    const int c = t / np, b = t - c * np;
    double v = 0.0;
    if (c < nq) {
      v = Vd[c + (size_t)nq * b];
    } else if (c < nq + nf) {
      const int j = c - nq;
      for (int q = op.R_ptr[j]; q < op.R_ptr[j + 1]; ++q) v = fma(-op.R_val[q], Vd[op.R_idx[q] + (size_t)nq * b], v);
    }
    M[t] = v;
  }
}

// E_k = A_k M for element k = blockIdx.x in FP64 (A_k column-major, staged in
// shared memory), rounded to FP32 in column quads: float4 (q, r) holds
// E_k[r, 4q .. 4q+3].
__global__ void __launch_bounds__(256) tail_operator_kernel(const double *__restrict__ Ak,
                                                            const double *__restrict__ M, float4 *__restrict__ E,
                                                            int np, int quads) {
  extern __shared__ double a_s[];
  const size_t k = blockIdx.x;
  const double *A = Ak + k * np * np;
  for (int t = threadIdx.x; t < np * np; t += blockDim.x) a_s[t] = A[t];
  __syncthreads();
  float4 *Ek = E + k * quads * np;
  for (int t = threadIdx.x; t < quads * np; t += blockDim.x) {
    const int q = t / np, r = t - q * np;
    const double *m0 = M + (size_t)(4 * q) * np;
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    for (int b = 0; b < np; ++b) {
      const double a = a_s[b * np + r];
      s0 = fma(a, m0[b], s0);
      s1 = fma(a, m0[np + b], s1);
      s2 = fma(a, m0[2 * np + b], s2);
      s3 = fma(a, m0[3 * np + b], s3);
    }
    Ek[t] = make_float4((float)s0, (float)s1, (float)s2, (float)s3);
  }
}

cudaError_t launch_tail_operators(const KernelArgs &ka, const double *Vd, double *M, float *E, int quads,
                                  cudaStream_t st) {
  const int np = ka.op.np, ncol = 4 * quads;
  tail_matrix_kernel<<<(np * ncol + 255) / 256, 256, 0, st>>>(ka.op, Vd, M, ncol);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  const size_t sm = (size_t)np * np * sizeof(double);
  if ((e = cudaFuncSetAttribute((const void *)tail_operator_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)sm)))
    return e;
  tail_operator_kernel<<<ka.ne, 256, sm, st>>>(ka.Ak, M, reinterpret_cast<float4 *>(E), np, quads);
  return cudaGetLastError();
}

cudaError_t launch_rk4_stage(const double *u, double *ust, double *acc, const double *k, double acc_w,
                             double c, int first, size_t n, cudaStream_t st) {
  rk4_stage_kernel<<<elementwise_grid(n), 256, 0, st>>>(u, ust, acc, k, acc_w, c, first, n);
  return cudaGetLastError();
}

cudaError_t launch_rk4_final(double *u, const double *acc, const double *k, double dt6, size_t n,
                             cudaStream_t st) {
  rk4_final_kernel<<<elementwise_grid(n), 256, 0, st>>>(u, acc, k, dt6, n);
  return cudaGetLastError();
}

cudaError_t launch_facet_layout(const double *in, double *out, int nf, int ne, int nc, cudaStream_t st) {
  size_t n = (size_t)nf * ne * nc;
  facet_to_reference_layout<<<elementwise_grid(n), 256, 0, st>>>(in, out, nf, ne, nc);
  return cudaGetLastError();
}

}  // namespace sse
