// sse_adjoint.cu -- discrete adjoint of the FP64 flux-differencing residual
// (Euler, entropy-conservative volume flux, Lax-Friedrichs or EC interface
// flux): mu = (dR/du)^T lam for the residual of flux_differencing_form.jl:
// 253-347, with no counterpart in the reference (which has no AD).
//
// Three kernels per vector-Jacobian product, after the forward phase A has
// written u_q, u_f for the state:
//   adj_lift_kernel     rbar_q = V M lam, interface cotangent gbar = -BJf R rbar_q
//   adj_flux_kernel     per-pair transposes of the contracted EC flux, the
//                       interface flux seen from both sides (no cross-element
//                       atomics: each element differentiates its own flux
//                       w.r.t. its inner state and its neighbour's flux w.r.t.
//                       the neighbour's outer state), deterministic chunked
//                       two-pass accumulation -> ubar_q, ubar_f
//   adj_projection_kernel  recomputes the entropy projection and applies its
//                       transpose (symmetric Jacobians of the entropy maps) -> mu
#include "sse_device.cuh"
#include "sse_kernels.cuh"
#include "sse_ops.cuh"

namespace sse {

// ---------------------------------------------------------------------------
template <int D, int NC>
__global__ void __launch_bounds__(256) adj_lift_kernel(KernelArgs ka) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Layout &L = ka.layAdjB1;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq, nf = op.nf;
  double *base = smem + (size_t)team * L.team_doubles;
  double *X = base + L.off[0], *Y = base + L.off[1], *Z = base + L.off[2], *Wb = base + L.off[3],
         *F = base + L.off[4];
  const double *lk = ka.lam + (size_t)kk * NC * np;
  for (int t = lane; t < NC * np; t += tpe) X[t] = lk[t];
  __syncthreads();
  // dudt = M V^T r_q  =>  rbar_q = V M^T lam (M symmetric)
  mass_solve<double, D, NC>(op, ka.geo.JinvW ? ka.geo.JinvW + (size_t)kk * nq : nullptr,
                            ka.geo.WJinv ? ka.geo.WJinv + (size_t)kk * nq : nullptr, ka.mass_wa, X, Y,
                            Z, Wb, lane, tpe);
  vdm_mul<double, D, NC>(op, X, Y, Z, Wb, lane, tpe);
  if (live)
    for (int t = lane; t < NC * nq; t += tpe) ka.rbar_q[(size_t)kk * NC * nq + t] = Y[t];
  // r_q -= R^T f_f  =>  fbar_f = -R rbar_q ; f_f = BJf f*  =>  gbar = BJf fbar_f
  csr_mul<double, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_val, Y, F, lane, tpe);
  __syncthreads();
  if (live)
    for (int t = lane; t < NC * nf; t += tpe)
      ka.gbar_f[(size_t)kk * NC * nf + t] = -F[t] * ka.geo.BJf[(size_t)kk * nf + t % nf];
}

// ---------------------------------------------------------------------------
// transpose of the Lax-Friedrichs interface flux
//   f* = ECdot(P(u_in), P(u_out), n) + a (u_in - u_out),
//   a = halfλ (max(|V_in.n|, |V_out.n|) + max(c_in, c_out)),
// with respect to one side: side = 0 inner, 1 outer.  Adds to Pb (primitive
// cotangent of that side) and ub_direct (cotangent of its conservative state
// through the a (u_in - u_out) term).
template <int D, int NC>
__device__ void lf_flux_bwd(const Physics &ph, const double *uin, const double *uout,
                            const double *Pin, const double *Pout, const double *n, const double *g,
                            int side, double *Pb, double *ub_direct) {
  double Pbi[3 + D], Pbo[3 + D];
  ec_flux_dot_bwd<D>(ph.igm1, Pin, Pout, n, g, Pbi, Pbo);
  const double *Pself = side ? Pbo : Pbi;
#pragma unroll
  for (int c = 0; c < 3 + D; ++c) Pb[c] += Pself[c];
  if (ph.nflux != 0) return;
  double vni = 0.0, vno = 0.0;
#pragma unroll
  for (int m = 0; m < D; ++m) { vni = fma(Pin[3 + m], n[m], vni); vno = fma(Pout[3 + m], n[m], vno); }
  const double ci = sqrt(ph.gamma * Pin[1] * sse_rcp(Pin[0]));
  const double co = sqrt(ph.gamma * Pout[1] * sse_rcp(Pout[0]));
  const double a = ph.half_lambda * (fmax(fabs(vni), fabs(vno)) + fmax(ci, co));
  double abar = 0.0;
#pragma unroll
  for (int e = 0; e < NC; ++e) {
    abar = fma(g[e], uin[e] - uout[e], abar);
    ub_direct[e] += side ? -a * g[e] : a * g[e];
  }
  const double hb = ph.half_lambda * abar;
  // max(|vni|, |vno|): the inner side owns ties (fmax returns its first argument's value)
  const bool v_in = fabs(vni) >= fabs(vno);
  const bool c_in = ci >= co;
  if (v_in == (side == 0)) {
    const double vn = side ? vno : vni;
    const double sg = vn >= 0.0 ? 1.0 : -1.0;
#pragma unroll
    for (int m = 0; m < D; ++m) Pb[3 + m] += hb * sg * n[m];
  }
  if (c_in == (side == 0)) {
    const double *P = side ? Pout : Pin;
    const double c = side ? co : ci;
    Pb[1] += hb * ph.gamma / (2.0 * c * P[0]);
    Pb[0] -= hb * c / (2.0 * P[0]);
  }
}

template <int D, int NC>
__global__ void __launch_bounds__(256) adj_flux_kernel(KernelArgs ka) {
  static_assert(NC == D + 2, "adjoint of the Euler flux-differencing residual");
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const DevGeo &g = ka.geo;
  const Layout &L = ka.layAdjB2;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int nq = op.nq, nf = op.nf, nfac = op.nfac, npf = op.npf;
  const int PS = 3 + D;
  double *base = smem + (size_t)team * L.team_doubles;
  double *uq = base + L.off[0], *uf = base + L.off[1], *rb = base + L.off[2], *fb = base + L.off[3],
         *prim = base + L.off[4], *Pb = base + L.off[5], *ubd = base + L.off[6], *Lam = base + L.off[7],
         *hnq = base + L.off[8], *buf = base + L.off[9];

  for (int t = lane; t < NC * nq; t += tpe) {
    uq[t] = ka.u_q[(size_t)kk * NC * nq + t];
    rb[t] = ka.rbar_q[(size_t)kk * NC * nq + t];
  }
  for (int t = lane; t < NC * nf; t += tpe) {
    uf[t] = ka.u_f[(size_t)kk * NC * nf + t];
    ubd[t] = 0.0;
  }
  for (int t = lane; t < nq * D * D; t += tpe) Lam[t] = g.Lambda_q[(size_t)kk * nq * D * D + t];
  if (op.nfp > 0)
    for (int t = lane; t < D * nfac * nq; t += tpe) hnq[t] = g.halfnJq[(size_t)kk * D * nfac * nq + t];
  for (int t = lane; t < (nq + nf) * PS; t += tpe) Pb[t] = 0.0;
  __syncthreads();
  for (int i = lane; i < nq + nf; i += tpe) {
    double u[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) u[e] = (i < nq) ? uq[e * nq + i] : uf[e * nf + (i - nq)];
    euler_prim_fast<D>(ph.gm1, u, prim + (size_t)i * PS);
  }
  // fbar_f = -R rbar_q
  csr_mul<double, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_val, rb, fb, lane, tpe);
  __syncthreads();
  for (int t = lane; t < NC * nf; t += tpe) fb[t] = -fb[t];

  // interface flux: own flux w.r.t. the inner state, neighbour's flux w.r.t. its outer state
  for (int j = lane; j < nf; j += tpe) {
    const int P = g.mapP[(size_t)kk * nf + j];
    const int jn = P % nf, kn = P / nf;
    double ui[NC], uo[NC], Po[3 + D], n[D], nn[D], gown[NC], gnb[NC], ub[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      ui[e] = uf[e * nf + j];
      uo[e] = ka.u_f[((size_t)kn * NC + e) * nf + jn];
      gown[e] = ka.gbar_f[((size_t)kk * NC + e) * nf + j];
      gnb[e] = ka.gbar_f[((size_t)kn * NC + e) * nf + jn];
      ub[e] = 0.0;
    }
#pragma unroll
    for (int m = 0; m < D; ++m) {
      n[m] = g.n_f[m + D * (j + (size_t)nf * kk)];
      nn[m] = g.n_f[m + D * (jn + (size_t)nf * kn)];
    }
    euler_prim_fast<D>(ph.gm1, uo, Po);
    double *Pself = Pb + (size_t)(nq + j) * PS;
    const double *Pi = prim + (size_t)(nq + j) * PS;
    lf_flux_bwd<D, NC>(ph, ui, uo, Pi, Po, n, gown, 0, Pself, ub);
    lf_flux_bwd<D, NC>(ph, uo, ui, Po, Pi, nn, gnb, 1, Pself, ub);
#pragma unroll
    for (int e = 0; e < NC; ++e) ubd[e * nf + j] += ub[e];
  }
  __syncthreads();

  // volume pairs: dbar_p = rbar[j] - rbar[i]; each node keeps a cursor into
  // its (ascending) incidence list across the chunks
  const int CH = ka.pair_chunk;
  int cur[kMaxNodeSlots];
#pragma unroll
  for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
    const int i = lane + sl * tpe;
    cur[sl] = i < nq ? op.vp_inc_ptr[i] : 0;
  }
  for (int c0 = 0; c0 < op.nvp; c0 += CH) {
    const int c1 = min(op.nvp, c0 + CH);
    for (int pidx = c0 + lane; pidx < c1; pidx += tpe) {
      const int ij = op.vp_ij[pidx];
      const int i = ij & 0xffff, j = ij >> 16;
      double G[D], db[NC];
#pragma unroll
      for (int n_ = 0; n_ < D; ++n_) G[n_] = 0.0;
#pragma unroll
      for (int m = 0; m < D; ++m) {
        const double Sm = op.vp_S[pidx * D + m];
        if (Sm == 0.0) continue;
#pragma unroll
        for (int n_ = 0; n_ < D; ++n_)
          G[n_] = fma(Sm, Lam[i + nq * (m + D * n_)] + Lam[j + nq * (m + D * n_)], G[n_]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) db[e] = rb[e * nq + j] - rb[e * nq + i];
      double *slot = buf + (size_t)(pidx - c0) * 2 * PS;
      ec_flux_dot_bwd<D>(ph.igm1, prim + (size_t)i * PS, prim + (size_t)j * PS, G, db, slot, slot + PS);
    }
    __syncthreads();
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int i = lane + sl * tpe;
      if (i >= nq) continue;
      double acc[3 + D];
#pragma unroll
      for (int c = 0; c < PS; ++c) acc[c] = 0.0;
      int q = cur[sl];
      const int qe = op.vp_inc_ptr[i + 1];
      for (; q < qe; ++q) {
        const int inc = op.vp_inc[q];
        const int pidx = inc >> 1;
        if (pidx >= c1) break;
        const double *slot = buf + (size_t)(pidx - c0) * 2 * PS + ((inc & 1) ? 0 : PS);
#pragma unroll
        for (int c = 0; c < PS; ++c) acc[c] += slot[c];
      }
      cur[sl] = q;
#pragma unroll
      for (int c = 0; c < PS; ++c) Pb[(size_t)i * PS + c] += acc[c];
    }
    __syncthreads();
  }

  // facet correction pairs: dbar_p = -rbar[i] - fbar_f[j]
  if (op.nfp > 0) {
    const double *hnf = g.halfnJf + (size_t)kk * D * nf;
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int t = lane + sl * tpe;
      cur[sl] = t < nq ? op.fp_q_ptr[t] : (t < nq + nf ? op.fp_f_ptr[t - nq] : 0);
    }
    for (int c0 = 0; c0 < op.nfp; c0 += CH) {
      const int c1 = min(op.nfp, c0 + CH);
      for (int pidx = c0 + lane; pidx < c1; pidx += tpe) {
        const int ij = op.fp_ij[pidx];
        const int i = ij & 0xffff, j = ij >> 16;
        const int f = j / npf;
        const double Cij = op.fp_C[pidx];
        double G[D], db[NC];
#pragma unroll
        for (int m = 0; m < D; ++m) G[m] = Cij * (hnf[m + D * j] + hnq[m + D * (f + nfac * i)]);
#pragma unroll
        for (int e = 0; e < NC; ++e) db[e] = -rb[e * nq + i] - fb[e * nf + j];
        double *slot = buf + (size_t)(pidx - c0) * 2 * PS;
        ec_flux_dot_bwd<D>(ph.igm1, prim + (size_t)i * PS, prim + (size_t)(nq + j) * PS, G, db, slot,
                           slot + PS);
      }
      __syncthreads();
#pragma unroll
      for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
        const int t = lane + sl * tpe;
        if (t >= nq + nf) continue;
        const bool vol = t < nq;
        const int r = vol ? t : t - nq;
        const int *lst = vol ? op.fp_q : op.fp_f;
        const int qe = vol ? op.fp_q_ptr[r + 1] : op.fp_f_ptr[r + 1];
        double acc[3 + D];
#pragma unroll
        for (int c = 0; c < PS; ++c) acc[c] = 0.0;
        int q = cur[sl];
        for (; q < qe; ++q) {
          const int pidx = lst[q];
          if (pidx >= c1) break;
          const double *slot = buf + (size_t)(pidx - c0) * 2 * PS + (vol ? 0 : PS);
#pragma unroll
          for (int c = 0; c < PS; ++c) acc[c] += slot[c];
        }
        cur[sl] = q;
#pragma unroll
        for (int c = 0; c < PS; ++c) Pb[(size_t)t * PS + c] += acc[c];
      }
      __syncthreads();
    }
  }

  // primitive cotangents -> conservative cotangents of u_q and u_f
  if (live) {
    for (int t = lane; t < nq + nf; t += tpe) {
      const bool vol = t < nq;
      const int r = vol ? t : t - nq;
      double u[NC], ub[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        u[e] = vol ? uq[e * nq + r] : uf[e * nf + r];
        ub[e] = vol ? 0.0 : ubd[e * nf + r];
      }
      euler_prim_bwd<D>(ph.gm1, u, prim + (size_t)t * PS, Pb + (size_t)t * PS, ub);
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        if (vol) ka.ubar_q[(size_t)kk * NC * nq + e * nq + r] = ub[e];
        else ka.ubar_f[((size_t)kk * NC + e) * nf + r] = ub[e];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// transpose of the entropy projection (flux_differencing_form.jl:190-250)
template <int D, int NC>
__global__ void __launch_bounds__(256) adj_projection_kernel(KernelArgs ka) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const Layout &L = ka.layAdjA;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq, nf = op.nf;
  double *base = smem + (size_t)team * L.team_doubles;
  double *X = base + L.off[0], *Y = base + L.off[1], *Z = base + L.off[2], *Wb = base + L.off[3],
         *F = base + L.off[4], *Uq0 = base + L.off[5], *Wq = base + L.off[6], *Wf = base + L.off[7],
         *Bq = base + L.off[8], *Bf = base + L.off[9];
  const double *WJ = ka.geo.WJ + (size_t)kk * nq;
  const double *JinvW = ka.geo.JinvW ? ka.geo.JinvW + (size_t)kk * nq : nullptr;

  // ---- forward recompute
  for (int t = lane; t < NC * np; t += tpe) X[t] = ka.u[(size_t)kk * NC * np + t];
  __syncthreads();
  vdm_mul<double, D, NC>(op, X, Uq0, Z, Wb, lane, tpe);  // u_q0 = V u (= u for nodal)
  for (int i = lane; i < nq; i += tpe) {
    double ui[NC], wi[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) ui[e] = Uq0[e * nq + i];
    cons_to_entropy_fast<D>(ph.gamma, ph.gm1, ph.igm1, ui, wi);
    const double s = op.has_vdm ? WJ[i] : 1.0;
#pragma unroll
    for (int e = 0; e < NC; ++e) X[e * nq + i] = wi[e] * s;
  }
  __syncthreads();
  if (op.has_vdm) {
    vdm_tmul<double, D, NC>(op, X, F, Z, Wb, lane, tpe);
    mass_solve<double, D, NC>(op, JinvW, nullptr, 1, F, X, Z, Wb, lane, tpe);
    vdm_mul<double, D, NC>(op, F, Wq, Z, Wb, lane, tpe);  // projected w_q
  } else {
    for (int t = lane; t < NC * nq; t += tpe) Wq[t] = X[t];
    __syncthreads();
  }
  csr_mul<double, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_val, Wq, Wf, lane, tpe);
  for (int t = lane; t < NC * nq; t += tpe) Bq[t] = ka.ubar_q[(size_t)kk * NC * nq + t];
  for (int t = lane; t < NC * nf; t += tpe) Bf[t] = ka.ubar_f[(size_t)kk * NC * nf + t];
  __syncthreads();

  // ---- backward
  // facet: wbar_f = J_e2c(w_f)^T ubar_f
  for (int j = lane; j < nf; j += tpe) {
    double wi[NC], bi[NC], ri[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) { wi[e] = Wf[e * nf + j]; bi[e] = Bf[e * nf + j]; }
    entropy_to_cons_jvp<D>(ph.gamma, ph.gm1, ph.igm1, ph.log_gm1, wi, bi, ri);
#pragma unroll
    for (int e = 0; e < NC; ++e) Bf[e * nf + j] = ri[e];
  }
  if (op.has_vdm) {
    // volume: wbar_q = J_e2c(w_q)^T ubar_q
    for (int i = lane; i < nq; i += tpe) {
      double wi[NC], bi[NC], ri[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) { wi[e] = Wq[e * nq + i]; bi[e] = Bq[e * nq + i]; }
      entropy_to_cons_jvp<D>(ph.gamma, ph.gm1, ph.igm1, ph.log_gm1, wi, bi, ri);
#pragma unroll
      for (int e = 0; e < NC; ++e) Bq[e * nq + i] = ri[e];
    }
  }
  __syncthreads();
  // wbar_q += R^T wbar_f   (into Y)
  for (int t = lane; t < NC * nq; t += tpe) {
    const int i = t % nq, e = t / nq;
    double acc = 0.0;
    for (int q = op.Rt_ptr[i]; q < op.Rt_ptr[i + 1]; ++q) acc += op.Rt_val[q] * Bf[e * nf + op.Rt_idx[q]];
    Y[t] = op.has_vdm ? Bq[t] + acc : acc;
  }
  __syncthreads();
  if (op.has_vdm) {
    // w_q = V M V^T (WJ c2e(u_q0))  =>  wbar_c2e = WJ .* V M V^T wbar_q
    vdm_tmul<double, D, NC>(op, Y, F, Z, Wb, lane, tpe);
    mass_solve<double, D, NC>(op, JinvW, nullptr, 1, F, X, Z, Wb, lane, tpe);
    vdm_mul<double, D, NC>(op, F, Y, Z, Wb, lane, tpe);
    for (int t = lane; t < NC * nq; t += tpe) Y[t] *= WJ[t % nq];
    __syncthreads();
  }
  // ubar_q0 = J_c2e(u_q0)^T wbar
  for (int i = lane; i < nq; i += tpe) {
    double ui[NC], bi[NC], ri[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) { ui[e] = Uq0[e * nq + i]; bi[e] = Y[e * nq + i]; }
    cons_to_entropy_jvp<D>(ph.gamma, ph.gm1, ph.igm1, ui, bi, ri);
#pragma unroll
    for (int e = 0; e < NC; ++e) Y[e * nq + i] = op.has_vdm ? ri[e] : ri[e] + Bq[e * nq + i];
  }
  __syncthreads();
  vdm_tmul<double, D, NC>(op, Y, F, Z, Wb, lane, tpe);  // mu = V^T ubar_q0
  if (live)
    for (int t = lane; t < NC * np; t += tpe) ka.mu[(size_t)kk * NC * np + t] = F[t];
}

// ===========================================================================
// Mixed-form vector-Jacobian product: the transposes of the mixed residual
// (FP32 fluxes on perturbations, FP32 projection arithmetic), with the
// cotangent of the reduced residual lam~ = (lam_rho + H_ref lam_E, lam_m,
// lam_E).  The FP32 buffers live in the FP64 VJP scratch (reinterpreted).
// ===========================================================================

template <int D, int NC>
__global__ void __launch_bounds__(256) adj_lift_mixed_kernel(KernelArgs ka) {
  extern __shared__ double smem_raw[];
  float *smem = reinterpret_cast<float *>(smem_raw);
  const DevOps &op = ka.op;
  const Layout &L = ka.layAdjB1m;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq, nf = op.nf;
  float *base = smem + (size_t)team * L.team_doubles;  // floats
  float *X = base + L.off[0], *Y = base + L.off[1], *Z = base + L.off[2], *Wb = base + L.off[3],
        *F = base + L.off[4];
  const double *lk = ka.lam + (size_t)kk * NC * np;
  for (int t = lane; t < NC * np; t += tpe) {
    const int e = t / np;
    const double v = (e == 0) ? fma(ka.ph.H_ref, lk[t + (NC - 1) * np], lk[t]) : lk[t];
    X[t] = (float)v;
  }
  __syncthreads();
  mass_solve<float, D, NC>(op, ka.geo.JinvWf ? ka.geo.JinvWf + (size_t)kk * nq : nullptr,
                           ka.geo.WJinvf ? ka.geo.WJinvf + (size_t)kk * nq : nullptr, ka.mass_wa, X, Y, Z,
                           Wb, lane, tpe);
  vdm_mul<float, D, NC>(op, X, Y, Z, Wb, lane, tpe);
  float *rbq = reinterpret_cast<float *>(ka.rbar_q);
  float *gbf = reinterpret_cast<float *>(ka.gbar_f);
  if (live)
    for (int t = lane; t < NC * nq; t += tpe) rbq[(size_t)kk * NC * nq + t] = Y[t];
  csr_mul<float, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_valf, Y, F, lane, tpe);
  __syncthreads();
  if (live)
    for (int t = lane; t < NC * nf; t += tpe)
      gbf[(size_t)kk * NC * nf + t] = -F[t] * ka.geo.BJff[(size_t)kk * nf + t % nf];
}

// transpose of the mixed-form Lax-Friedrichs interface flux w.r.t. one side
// (reduced energy: the jump's energy component is E' - H_ref rho')
template <int D, int NC>
__device__ void lf_flux_mixed_bwd(const Physics &ph, float igm1, float rho_ref, float theta_ref, float H_ref,
                                  const float *uin, const float *uout, const float *Pin, const float *Pout,
                                  const float *n, const float *g, int side, float *Pb, float *ub_direct) {
  float Pbi[4 + D], Pbo[4 + D];
  ec_flux_dot_mixed_bwd<D>(igm1, rho_ref, theta_ref, Pin, Pout, n, g, Pbi, Pbo);
  const float *Pself = side ? Pbo : Pbi;
#pragma unroll
  for (int c = 0; c < 4 + D; ++c) Pb[c] += Pself[c];
  if (ph.nflux != 0) return;
  const float hl = (float)ph.half_lambda, gam = (float)ph.gamma;
  float vni = 0.f, vno = 0.f;
#pragma unroll
  for (int m = 0; m < D; ++m) { vni = fmaf(Pin[3 + m], n[m], vni); vno = fmaf(Pout[3 + m], n[m], vno); }
  const float ci = sqrtf(gam * (theta_ref + Pin[2])), co = sqrtf(gam * (theta_ref + Pout[2]));
  const float a = hl * (fmaxf(fabsf(vni), fabsf(vno)) + fmaxf(ci, co));
  float abar = 0.f;
#pragma unroll
  for (int e = 0; e < NC; ++e) abar = fmaf(g[e], uin[e] - uout[e], abar);
  abar = fmaf(-H_ref * g[NC - 1], uin[0] - uout[0], abar);
  const float sg_side = side ? -1.f : 1.f;
#pragma unroll
  for (int e = 0; e < NC; ++e) ub_direct[e] += sg_side * a * g[e];
  ub_direct[0] -= sg_side * a * H_ref * g[NC - 1];
  const float hb = hl * abar;
  const bool v_in = fabsf(vni) >= fabsf(vno);
  const bool c_in = ci >= co;
  if (v_in == (side == 0)) {
    const float vn = side ? vno : vni;
    const float sg = vn >= 0.f ? 1.f : -1.f;
#pragma unroll
    for (int m = 0; m < D; ++m) Pb[3 + m] += hb * sg * n[m];
  }
  if (c_in == (side == 0)) {
    const float c = side ? co : ci;
    Pb[2] += hb * gam / (2.f * c);
  }
}

template <int D, int NC>
__global__ void __launch_bounds__(256) adj_flux_mixed_kernel(KernelArgs ka) {
  static_assert(NC == D + 2, "adjoint of the Euler flux-differencing residual");
  extern __shared__ double smem_raw[];
  float *smem = reinterpret_cast<float *>(smem_raw);
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const DevGeo &g = ka.geo;
  const Layout &L = ka.layAdjB2m;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int nq = op.nq, nf = op.nf, nfac = op.nfac, npf = op.npf;
  const int PS = 4 + D;
  const float gm1 = (float)ph.gm1, igm1 = (float)ph.igm1;
  const float rho_ref = (float)ph.rho_ref, p_ref = (float)ph.p_ref;
  const float theta_ref = (float)ph.theta_ref, H_ref = (float)ph.H_ref;
  float *base = smem + (size_t)team * L.team_doubles;
  float *uq = base + L.off[0], *uf = base + L.off[1], *rb = base + L.off[2], *fb = base + L.off[3],
        *prim = base + L.off[4], *Pb = base + L.off[5], *ubd = base + L.off[6], *Lam = base + L.off[7],
        *hnq = base + L.off[8], *buf = base + L.off[9];
  const float *rbq = reinterpret_cast<const float *>(ka.rbar_q);
  const float *gbf = reinterpret_cast<const float *>(ka.gbar_f);

  for (int t = lane; t < NC * nq; t += tpe) {
    uq[t] = ka.u_qf[(size_t)kk * NC * nq + t];
    rb[t] = rbq[(size_t)kk * NC * nq + t];
  }
  for (int t = lane; t < NC * nf; t += tpe) {
    uf[t] = ka.u_ff[(size_t)kk * NC * nf + t];
    ubd[t] = 0.f;
  }
  for (int t = lane; t < nq * D * D; t += tpe) Lam[t] = g.Lambda_qf[(size_t)kk * nq * D * D + t];
  // halfnJq is staged when the layout has room for it, else read from global
  // memory (the host drops it from the layout to keep more blocks per SM)
  const float *hnq_src = hnq;
  if (op.nfp > 0) {
    if (L.off[9] > L.off[8]) {
      for (int t = lane; t < D * nfac * nq; t += tpe) hnq[t] = g.halfnJqf[(size_t)kk * D * nfac * nq + t];
    } else {
      hnq_src = g.halfnJqf + (size_t)kk * D * nfac * nq;
    }
  }
  for (int t = lane; t < (nq + nf) * PS; t += tpe) Pb[t] = 0.f;
  __syncthreads();
  for (int i = lane; i < nq + nf; i += tpe) {
    float du[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) du[e] = (i < nq) ? uq[e * nq + i] : uf[e * nf + (i - nq)];
    euler_prim_mixed<D>(gm1, rho_ref, p_ref, du, prim + (size_t)i * PS);
  }
  csr_mul<float, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_valf, rb, fb, lane, tpe);
  __syncthreads();
  for (int t = lane; t < NC * nf; t += tpe) fb[t] = -fb[t];

  // interface flux: own flux w.r.t. the inner state, neighbour's w.r.t. its outer state
  for (int j = lane; j < nf; j += tpe) {
    const int P = g.mapP[(size_t)kk * nf + j];
    const int jn = P % nf, kn = P / nf;
    float ui[NC], uo[NC], Po[4 + D], n[D], nn[D], gown[NC], gnb[NC], ub[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      ui[e] = uf[e * nf + j];
      uo[e] = ka.u_ff[((size_t)kn * NC + e) * nf + jn];
      gown[e] = gbf[((size_t)kk * NC + e) * nf + j];
      gnb[e] = gbf[((size_t)kn * NC + e) * nf + jn];
      ub[e] = 0.f;
    }
#pragma unroll
    for (int m = 0; m < D; ++m) {
      n[m] = g.n_ff[m + D * (j + (size_t)nf * kk)];
      nn[m] = g.n_ff[m + D * (jn + (size_t)nf * kn)];
    }
    euler_prim_mixed<D>(gm1, rho_ref, p_ref, uo, Po);
    float *Pself = Pb + (size_t)(nq + j) * PS;
    const float *Pi = prim + (size_t)(nq + j) * PS;
    lf_flux_mixed_bwd<D, NC>(ph, igm1, rho_ref, theta_ref, H_ref, ui, uo, Pi, Po, n, gown, 0, Pself, ub);
    lf_flux_mixed_bwd<D, NC>(ph, igm1, rho_ref, theta_ref, H_ref, uo, ui, Po, Pi, nn, gnb, 1, Pself, ub);
#pragma unroll
    for (int e = 0; e < NC; ++e) ubd[e * nf + j] += ub[e];
  }
  __syncthreads();

  // volume pairs: dbar_p = rbar[j] - rbar[i]
  const int CH = ka.pair_chunk_mixed;
  const float *vpS = op.vp_Sf;
  int cur[kMaxNodeSlots];
#pragma unroll
  for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
    const int i = lane + sl * tpe;
    cur[sl] = i < nq ? op.vp_inc_ptr[i] : 0;
  }
  for (int c0 = 0; c0 < op.nvp; c0 += CH) {
    const int c1 = min(op.nvp, c0 + CH);
    for (int pidx = c0 + lane; pidx < c1; pidx += tpe) {
      const int ij = op.vp_ij[pidx];
      const int i = ij & 0xffff, j = ij >> 16;
      float G[D], db[NC];
#pragma unroll
      for (int n_ = 0; n_ < D; ++n_) G[n_] = 0.f;
#pragma unroll
      for (int m = 0; m < D; ++m) {
        const float Sm = vpS[pidx * D + m];
        if (Sm == 0.f) continue;
#pragma unroll
        for (int n_ = 0; n_ < D; ++n_)
          G[n_] = fmaf(Sm, Lam[i + nq * (m + D * n_)] + Lam[j + nq * (m + D * n_)], G[n_]);
      }
#pragma unroll
      for (int e = 0; e < NC; ++e) db[e] = rb[e * nq + j] - rb[e * nq + i];
      float *slot = buf + (size_t)(pidx - c0) * 2 * PS;
      ec_flux_dot_mixed_bwd<D>(igm1, rho_ref, theta_ref, prim + (size_t)i * PS, prim + (size_t)j * PS, G, db,
                               slot, slot + PS);
    }
    __syncthreads();
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int i = lane + sl * tpe;
      if (i >= nq) continue;
      float acc[4 + D];
#pragma unroll
      for (int c = 0; c < PS; ++c) acc[c] = 0.f;
      int q = cur[sl];
      const int qe = op.vp_inc_ptr[i + 1];
      for (; q < qe; ++q) {
        const int inc = op.vp_inc[q];
        const int pidx = inc >> 1;
        if (pidx >= c1) break;
        const float *slot = buf + (size_t)(pidx - c0) * 2 * PS + ((inc & 1) ? 0 : PS);
#pragma unroll
        for (int c = 0; c < PS; ++c) acc[c] += slot[c];
      }
      cur[sl] = q;
#pragma unroll
      for (int c = 0; c < PS; ++c) Pb[(size_t)i * PS + c] += acc[c];
    }
    __syncthreads();
  }

  // facet correction pairs: dbar_p = -rbar[i] - fbar_f[j]
  if (op.nfp > 0) {
    const float *hnf = g.halfnJff + (size_t)kk * D * nf;
    const float *fpC = op.fp_Cf;
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int t = lane + sl * tpe;
      cur[sl] = t < nq ? op.fp_q_ptr[t] : (t < nq + nf ? op.fp_f_ptr[t - nq] : 0);
    }
    for (int c0 = 0; c0 < op.nfp; c0 += CH) {
      const int c1 = min(op.nfp, c0 + CH);
      for (int pidx = c0 + lane; pidx < c1; pidx += tpe) {
        const int ij = op.fp_ij[pidx];
        const int i = ij & 0xffff, j = ij >> 16;
        const int f = j / npf;
        const float Cij = fpC[pidx];
        float G[D], db[NC];
#pragma unroll
        for (int m = 0; m < D; ++m) G[m] = Cij * (hnf[m + D * j] + hnq_src[m + D * (f + nfac * i)]);
#pragma unroll
        for (int e = 0; e < NC; ++e) db[e] = -rb[e * nq + i] - fb[e * nf + j];
        float *slot = buf + (size_t)(pidx - c0) * 2 * PS;
        ec_flux_dot_mixed_bwd<D>(igm1, rho_ref, theta_ref, prim + (size_t)i * PS, prim + (size_t)(nq + j) * PS,
                                 G, db, slot, slot + PS);
      }
      __syncthreads();
#pragma unroll
      for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
        const int t = lane + sl * tpe;
        if (t >= nq + nf) continue;
        const bool vol = t < nq;
        const int r = vol ? t : t - nq;
        const int *lst = vol ? op.fp_q : op.fp_f;
        const int qe = vol ? op.fp_q_ptr[r + 1] : op.fp_f_ptr[r + 1];
        float acc[4 + D];
#pragma unroll
        for (int c = 0; c < PS; ++c) acc[c] = 0.f;
        int q = cur[sl];
        for (; q < qe; ++q) {
          const int pidx = lst[q];
          if (pidx >= c1) break;
          const float *slot = buf + (size_t)(pidx - c0) * 2 * PS + (vol ? 0 : PS);
#pragma unroll
          for (int c = 0; c < PS; ++c) acc[c] += slot[c];
        }
        cur[sl] = q;
#pragma unroll
        for (int c = 0; c < PS; ++c) Pb[(size_t)t * PS + c] += acc[c];
      }
      __syncthreads();
    }
  }

  // primitive cotangents -> cotangents of the stored perturbations u_q', u_f'
  float *ubq = reinterpret_cast<float *>(ka.ubar_q);
  float *ubf = reinterpret_cast<float *>(ka.ubar_f);
  if (live) {
    for (int t = lane; t < nq + nf; t += tpe) {
      const bool vol = t < nq;
      const int r = vol ? t : t - nq;
      float ub[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) ub[e] = vol ? 0.f : ubd[e * nf + r];
      euler_prim_mixed_bwd<D>(gm1, theta_ref, prim + (size_t)t * PS, Pb + (size_t)t * PS, ub);
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        if (vol) ubq[(size_t)kk * NC * nq + e * nq + r] = ub[e];
        else ubf[((size_t)kk * NC + e) * nf + r] = ub[e];
      }
    }
  }
}

// transpose of the mixed-form entropy projection (nodal_values_mixed_kernel)
template <int D, int NC>
__global__ void __launch_bounds__(256) adj_projection_mixed_kernel(KernelArgs ka) {
  static_assert(NC == D + 2, "mixed form of the Euler entropy projection");
  extern __shared__ double smem_raw[];
  float *smem = reinterpret_cast<float *>(smem_raw);
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const Layout &L = ka.layAdjAm;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int np = op.np, nq = op.nq, nf = op.nf;
  float *base = smem + (size_t)team * L.team_doubles;
  float *U1 = base + L.off[0], *Q0 = base + L.off[1], *XQ = base + L.off[2], *WQ = base + L.off[3],
        *WF = base + L.off[4], *T1 = base + L.off[5], *S1 = base + L.off[6], *Zf = base + L.off[7],
        *Wf = base + L.off[8], *BF = base + L.off[9];
  const double *WJ = ka.geo.WJ + (size_t)kk * nq;
  const float *JinvWf = ka.geo.JinvWf + (size_t)kk * nq;
  const double *P1 = ka.geo.P1 + (size_t)kk * nq, *RP1 = ka.geo.RP1 + (size_t)kk * nf;

  // ---- forward recompute (as nodal_values_mixed_kernel)
  const double *uk = ka.u + (size_t)kk * NC * np;
  for (int t = lane; t < NC * np; t += tpe) {
    const int e = t / np, l = t - e * np;
    U1[t] = (float)(l == ph.mode0 ? uk[t] - ph.u_ref_modal[e] : uk[t]);
  }
  __syncthreads();
  vdm_mul<float, D, NC>(op, U1, Q0, Zf, Wf, lane, tpe);  // u_q0'
  for (int i = lane; i < nq; i += tpe) {
    double ui[NC], wi[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      const double ref = (e == 0) ? ph.rho_ref : ((e == NC - 1) ? ph.E_ref : 0.0);
      ui[e] = ref + (double)Q0[e * nq + i];
    }
    cons_to_entropy_mixed<D>(ph, ui, wi);
#pragma unroll
    for (int e = 0; e < NC; ++e) XQ[e * nq + i] = (float)(WJ[i] * (wi[e] - ph.w_ref[e]));
  }
  __syncthreads();
  vdm_tmul<float, D, NC>(op, XQ, T1, Zf, Wf, lane, tpe);
  mass_solve<float, D, NC>(op, JinvWf, nullptr, 1, T1, S1, Zf, Wf, lane, tpe);
  vdm_mul<float, D, NC>(op, T1, WQ, Zf, Wf, lane, tpe);                      // w'_q
  csr_mul<float, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_valf, WQ, WF, lane, tpe);  // w'_f
  __syncthreads();

  // ---- backward: facet then volume entropy-to-conservative transposes
  const float *ubq = reinterpret_cast<const float *>(ka.ubar_q);
  const float *ubf = reinterpret_cast<const float *>(ka.ubar_f);
  for (int t = lane; t < nq + nf; t += tpe) {
    const bool vol = t < nq;
    const int r = vol ? t : t - nq;
    const double p1 = vol ? P1[r] : RP1[r];
    const float *src = vol ? WQ + r : WF + r;
    const int stride = vol ? nq : nf;
    double wi[NC], bi[NC], ri[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      wi[e] = fma(ph.w_ref[e], p1, (double)src[e * stride]);
      bi[e] = vol ? (double)ubq[(size_t)kk * NC * nq + e * nq + r] : (double)ubf[((size_t)kk * NC + e) * nf + r];
    }
    const double rhoe = entropy_to_cons_mixed_rhoe<D>(ph, wi);
    entropy_to_cons_jvp_rhoe<D>(ph.gm1, ph.igm1, ph.gamma, wi, rhoe, bi, ri);
    float *dst = vol ? S1 + r : BF + r;
#pragma unroll
    for (int e = 0; e < NC; ++e) dst[e * stride] = (float)ri[e];
  }
  __syncthreads();
  // wbar_q += R^T wbar_f
  for (int t = lane; t < NC * nq; t += tpe) {
    const int i = t % nq, e = t / nq;
    float acc = 0.f;
    for (int q = op.Rt_ptr[i]; q < op.Rt_ptr[i + 1]; ++q) acc = fmaf(op.Rt_valf[q], BF[e * nf + op.Rt_idx[q]], acc);
    XQ[t] = S1[t] + acc;
  }
  __syncthreads();
  // projection transpose (V M V^T is symmetric): the same operators
  vdm_tmul<float, D, NC>(op, XQ, T1, Zf, Wf, lane, tpe);
  mass_solve<float, D, NC>(op, JinvWf, nullptr, 1, T1, S1, Zf, Wf, lane, tpe);
  vdm_mul<float, D, NC>(op, T1, XQ, Zf, Wf, lane, tpe);
  // ubar_q0 = J_c2e(u_q0)^T (W J x), symmetric Jacobian
  for (int i = lane; i < nq; i += tpe) {
    double ui[NC], bi[NC], ri[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      const double ref = (e == 0) ? ph.rho_ref : ((e == NC - 1) ? ph.E_ref : 0.0);
      ui[e] = ref + (double)Q0[e * nq + i];
      bi[e] = WJ[i] * (double)XQ[e * nq + i];
    }
    cons_to_entropy_jvp<D>(ph.gamma, ph.gm1, ph.igm1, ui, bi, ri);
#pragma unroll
    for (int e = 0; e < NC; ++e) XQ[e * nq + i] = (float)ri[e];
  }
  __syncthreads();
  vdm_tmul<float, D, NC>(op, XQ, T1, Zf, Wf, lane, tpe);  // mu = V^T ubar_q0
  if (live)
    for (int t = lane; t < NC * np; t += tpe) ka.mu[(size_t)kk * NC * np + t] = (double)T1[t];
}

// ---------------------------------------------------------------------------
// elementwise pieces of the adjoint Runge-Kutta sweep
//
// CarpenterKennedy2N54 stage s (forward: tmp = a_s tmp + dt k_s, u += b_s tmp,
// k_s = R(u_s)) reversed, with ybar the state adjoint and qbar the adjoint of
// tmp after the stage:
//   qbar += b_s ybar  (done by the previous reversal, or at the step's start)
//   ybar += dt (dR/du(u_s))^T qbar   <- mu
//   qbar  = a_s qbar + b_{s-1} ybar   (b_{-1} = 0, a_1 = 0 ends the step)
__global__ void adj_ck_stage_kernel(double *__restrict__ ybar, double *__restrict__ qbar,
                                    const double *__restrict__ mu, double dt, double a, double b_prev,
                                    size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double y = fma(dt, mu[i], ybar[i]);
    ybar[i] = y;
    qbar[i] = fma(a, qbar[i], b_prev * y);
  }
}

// y = beta x  (alpha == 0, y not read)  or  y = alpha y + beta x
__global__ void adj_lincomb_kernel(double *__restrict__ y, const double *__restrict__ x, double alpha,
                                   double beta, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
    y[i] = alpha == 0.0 ? beta * x[i] : fma(alpha, y[i], beta * x[i]);
}

// classic RK4 stage reversed: ybar += mu ; kbar = cy ybar' + cm mu (not on the last)
__global__ void adj_rk4_stage_kernel(double *__restrict__ ybar, double *__restrict__ kbar,
                                     const double *__restrict__ mu, const double *__restrict__ yp,
                                     double cy, double cm, int last, size_t n) {
  for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x) {
    const double m = mu[i];
    ybar[i] += m;
    if (!last) kbar[i] = fma(cy, yp[i], cm * m);
  }
}

static int grid_for(size_t n) {
  size_t g = (n + 255) / 256;
  return (int)(g > 152 * 16 ? 152 * 16 : (g < 1 ? 1 : g));
}

cudaError_t launch_adj_ck_stage(double *ybar, double *qbar, const double *mu, double dt, double a,
                                double b_prev, size_t n, cudaStream_t st) {
  adj_ck_stage_kernel<<<grid_for(n), 256, 0, st>>>(ybar, qbar, mu, dt, a, b_prev, n);
  return cudaGetLastError();
}

cudaError_t launch_adj_lincomb(double *y, const double *x, double alpha, double beta, size_t n,
                               cudaStream_t st) {
  adj_lincomb_kernel<<<grid_for(n), 256, 0, st>>>(y, x, alpha, beta, n);
  return cudaGetLastError();
}

cudaError_t launch_adj_rk4_stage(double *ybar, double *kbar, const double *mu, const double *yp,
                                 double cy, double cm, int last, size_t n, cudaStream_t st) {
  adj_rk4_stage_kernel<<<grid_for(n), 256, 0, st>>>(ybar, kbar, mu, yp, cy, cm, last, n);
  return cudaGetLastError();
}

cudaError_t sse_set_smem_limits_adjoint(const KernelArgs &ka) {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void *f, const Layout &L) {
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)((size_t)ka.epb * L.team_doubles * sizeof(double)));
  };
  if (ka.op.d == 2 && ka.op.nc == 4) {
    set((const void *)adj_lift_kernel<2, 4>, ka.layAdjB1);
    set((const void *)adj_flux_kernel<2, 4>, ka.layAdjB2);
    set((const void *)adj_projection_kernel<2, 4>, ka.layAdjA);
  } else if (ka.op.d == 3 && ka.op.nc == 5) {
    set((const void *)adj_lift_kernel<3, 5>, ka.layAdjB1);
    set((const void *)adj_flux_kernel<3, 5>, ka.layAdjB2);
    set((const void *)adj_projection_kernel<3, 5>, ka.layAdjA);
  } else {
    return cudaErrorInvalidValue;
  }
  return e;
}

cudaError_t sse_set_smem_limits_adjoint_mixed(const KernelArgs &ka) {
  cudaError_t e = cudaSuccess;
  auto set = [&](const void *f, const Layout &L) {
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               (int)((size_t)ka.epb * L.team_doubles * sizeof(float)));
  };
  if (ka.op.d == 2 && ka.op.nc == 4) {
    set((const void *)adj_lift_mixed_kernel<2, 4>, ka.layAdjB1m);
    set((const void *)adj_flux_mixed_kernel<2, 4>, ka.layAdjB2m);
    set((const void *)adj_projection_mixed_kernel<2, 4>, ka.layAdjAm);
  } else if (ka.op.d == 3 && ka.op.nc == 5) {
    set((const void *)adj_lift_mixed_kernel<3, 5>, ka.layAdjB1m);
    set((const void *)adj_flux_mixed_kernel<3, 5>, ka.layAdjB2m);
    set((const void *)adj_projection_mixed_kernel<3, 5>, ka.layAdjAm);
  } else {
    return cudaErrorInvalidValue;
  }
  return e;
}

cudaError_t launch_residual_vjp_mixed_kernels(const KernelArgs &ka, cudaStream_t st) {
  const int grid = (ka.ne + ka.epb - 1) / ka.epb;
  const size_t s1 = (size_t)ka.epb * ka.layAdjB1m.team_doubles * sizeof(float);
  const size_t s2 = (size_t)ka.epb * ka.layAdjB2m.team_doubles * sizeof(float);
  const size_t s3 = (size_t)ka.epb * ka.layAdjAm.team_doubles * sizeof(float);
  if (ka.op.d == 2 && ka.op.nc == 4) {
    adj_lift_mixed_kernel<2, 4><<<grid, ka.tpb, s1, st>>>(ka);
    adj_flux_mixed_kernel<2, 4><<<grid, ka.tpb, s2, st>>>(ka);
    adj_projection_mixed_kernel<2, 4><<<grid, ka.tpb, s3, st>>>(ka);
  } else if (ka.op.d == 3 && ka.op.nc == 5) {
    adj_lift_mixed_kernel<3, 5><<<grid, ka.tpb, s1, st>>>(ka);
    adj_flux_mixed_kernel<3, 5><<<grid, ka.tpb, s2, st>>>(ka);
    adj_projection_mixed_kernel<3, 5><<<grid, ka.tpb, s3, st>>>(ka);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

cudaError_t launch_residual_vjp_kernels(const KernelArgs &ka, cudaStream_t st) {
  const int grid = (ka.ne + ka.epb - 1) / ka.epb;
  const size_t s1 = (size_t)ka.epb * ka.layAdjB1.team_doubles * sizeof(double);
  const size_t s2 = (size_t)ka.epb * ka.layAdjB2.team_doubles * sizeof(double);
  const size_t s3 = (size_t)ka.epb * ka.layAdjA.team_doubles * sizeof(double);
  if (ka.op.d == 2 && ka.op.nc == 4) {
    adj_lift_kernel<2, 4><<<grid, ka.tpb, s1, st>>>(ka);
    adj_flux_kernel<2, 4><<<grid, ka.tpb, s2, st>>>(ka);
    adj_projection_kernel<2, 4><<<grid, ka.tpb, s3, st>>>(ka);
  } else if (ka.op.d == 3 && ka.op.nc == 5) {
    adj_lift_kernel<3, 5><<<grid, ka.tpb, s1, st>>>(ka);
    adj_flux_kernel<3, 5><<<grid, ka.tpb, s2, st>>>(ka);
    adj_projection_kernel<3, 5><<<grid, ka.tpb, s3, st>>>(ka);
  } else {
    return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace sse
