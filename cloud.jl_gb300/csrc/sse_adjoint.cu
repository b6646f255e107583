// sse_adjoint.cu -- discrete adjoint of the FP64 residual: mu = (dR/du)^T lam
// for every configuration of the forward -- FluxDifferencingForm
// (flux_differencing_form.jl:253-347) with the entropy-conservative or the
// conservative two-point flux, and StandardForm
// (standard_form_first_order.jl:1-63), for the Euler equations and linear
// advection, with any interface flux -- with no counterpart in the
// reference (which has no AD).
//
// Three kernels per vector-Jacobian product, after the forward phase A has
// written u_q, u_f for the state:
//   adj_lift_kernel     rbar_q = V M lam, interface cotangent gbar = -BJf R rbar_q
//   adj_flux_kernel     (Euler, EC flux) per-pair transposes of the contracted
//                       EC flux, the interface flux seen from both sides (no
//                       cross-element atomics: each element differentiates its
//                       own flux w.r.t. its inner state and its neighbour's
//                       flux w.r.t. the neighbour's outer state), deterministic
//                       chunked two-pass accumulation -> ubar_q, ubar_f
//   adj_flux_generic_kernel  the same for the conservative two-point flux
//   adj_std_flux_kernel      StandardForm volume, facet and interface transposes
//   adj_projection_kernel  (Euler FD) recomputes the entropy projection and
//                       applies its transpose (symmetric Jacobians of the
//                       entropy maps) -> mu
//   adj_nodal_kernel    (no projection) mu = V^T (ubar_q + R^T ubar_f)
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
                            Z, Wb, lane, tpe, ka.Ak ? ka.Ak + (size_t)kk * op.np * op.np : nullptr);
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
  const float rnpf = qrcp(npf > 0 ? npf : 1);
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
        const int f = qdiv(j, rnpf);
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
    cons_to_entropy_fast<D>(ph.gamma, ph.gm1, ph.igm1, ui, wi, ka.op.math_tab);
    const double s = op.has_vdm ? WJ[i] : 1.0;
#pragma unroll
    for (int e = 0; e < NC; ++e) X[e * nq + i] = wi[e] * s;
  }
  __syncthreads();
  if (op.has_vdm) {
    vdm_tmul<double, D, NC>(op, X, F, Z, Wb, lane, tpe);
    mass_solve<double, D, NC>(op, JinvW, nullptr, 1, F, X, Z, Wb, lane, tpe, ka.Ak ? ka.Ak + (size_t)kk * op.np * op.np : nullptr);
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
    entropy_to_cons_jvp<D>(ph.gamma, ph.gm1, ph.igm1, ph.log_gm1, wi, bi, ri, ka.op.math_tab);
#pragma unroll
    for (int e = 0; e < NC; ++e) Bf[e * nf + j] = ri[e];
  }
  if (op.has_vdm) {
    // volume: wbar_q = J_e2c(w_q)^T ubar_q
    for (int i = lane; i < nq; i += tpe) {
      double wi[NC], bi[NC], ri[NC];
#pragma unroll
      for (int e = 0; e < NC; ++e) { wi[e] = Wq[e * nq + i]; bi[e] = Bq[e * nq + i]; }
      entropy_to_cons_jvp<D>(ph.gamma, ph.gm1, ph.igm1, ph.log_gm1, wi, bi, ri, ka.op.math_tab);
#pragma unroll
      for (int e = 0; e < NC; ++e) Bq[e * nq + i] = ri[e];
    }
  }
  __syncthreads();
  // wbar_q += R^T wbar_f   (into Y)
  rt_apply<double, NC>(op, op.Rt_val, Bf, lane, tpe,
                       [&](int t, double v) { Y[t] = op.has_vdm ? Bq[t] + v : v; });
  __syncthreads();
  if (op.has_vdm) {
    // w_q = V M V^T (WJ c2e(u_q0))  =>  wbar_c2e = WJ .* V M V^T wbar_q
    vdm_tmul<double, D, NC>(op, Y, F, Z, Wb, lane, tpe);
    mass_solve<double, D, NC>(op, JinvW, nullptr, 1, F, X, Z, Wb, lane, tpe, ka.Ak ? ka.Ak + (size_t)kk * op.np * op.np : nullptr);
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
// StandardForm (standard_form_first_order.jl:1-63) and plain nodal values:
// after adj_lift_kernel,
//   adj_std_flux_kernel  transposes of the skew-symmetric volume terms
//                        (halfWΛ, D_m), the facet term -halfN R f_n, the
//                        physical flux and the interface numerical flux seen
//                        from both sides -> ubar_q, ubar_f
//   adj_nodal_kernel     u_q = V u, u_f = R u_q  =>  mu = V^T (ubar_q + R^T ubar_f)
// The same adj_nodal_kernel closes the FluxDifferencingForm VJP of scalar
// laws, which have no entropy projection.
// ===========================================================================

// Transpose of the physical flux F[e][n](u) (euler_navierstokes.jl:85-91;
// linear advection F[0][n] = a_n u) applied to Fb[e][n]; adds to ub.
template <int D, int NC>
__device__ __forceinline__ void physical_flux_vjp(const Physics &ph, const double *u,
                                                  const double (&Fb)[NC][D], double *ub) {
  if constexpr (NC == 1) {
#pragma unroll
    for (int n = 0; n < D; ++n) ub[0] = fma(ph.a[n], Fb[0][n], ub[0]);
  } else {
    const double ir = 1.0 / u[0];
    double V[D], vv = 0.0;
#pragma unroll
    for (int m = 0; m < D; ++m) { V[m] = u[m + 1] * ir; vv = fma(u[m + 1], V[m], vv); }
    const double p = ph.gm1 * (u[D + 1] - 0.5 * vv);
    const double ht = u[D + 1] + p;
    double Vb[D], pb = 0.0, htb = 0.0;
#pragma unroll
    for (int n = 0; n < D; ++n) {
      // F[0][n] = m_n ; F[m+1][n] = m_m V_n + delta_mn p ; F[D+1][n] = ht V_n
      ub[n + 1] += Fb[0][n];
      Vb[n] = Fb[D + 1][n] * ht;
      htb = fma(Fb[D + 1][n], V[n], htb);
      pb += Fb[n + 1][n];
#pragma unroll
      for (int m = 0; m < D; ++m) {
        ub[m + 1] = fma(Fb[m + 1][n], V[n], ub[m + 1]);
        Vb[n] = fma(Fb[m + 1][n], u[m + 1], Vb[n]);
      }
    }
    // ht = E + p ; p = gm1 (E - |m|^2 / (2 rho)) ; V = m / rho
    pb += htb;
    ub[D + 1] += htb + ph.gm1 * pb;
    double rb = 0.5 * ph.gm1 * pb * vv * ir;
#pragma unroll
    for (int m = 0; m < D; ++m) {
      ub[m + 1] += Vb[m] * ir - ph.gm1 * pb * V[m];
      rb -= Vb[m] * V[m] * ir;
    }
    ub[0] += rb;
  }
}

// Transpose, with respect to one side (0 inner, 1 outer), of the StandardForm
// interface flux f* = (F(u_in) + F(u_out))/2 . n + a (u_in - u_out) with
// a = halfλ wave_speed (LF; ConservationLaws.jl:75-128) or a = 0, applied to
// the cotangent g; adds to ub (that side's conservative cotangent).
template <int D, int NC>
__device__ void std_iface_bwd(const Physics &ph, const double *uin, const double *uout,
                              const double *n, const double *g, int side, double *ub) {
  const double *us = side ? uout : uin;
  double Fb[NC][D];
#pragma unroll
  for (int e = 0; e < NC; ++e)
#pragma unroll
    for (int m = 0; m < D; ++m) Fb[e][m] = 0.5 * g[e] * n[m];
  physical_flux_vjp<D, NC>(ph, us, Fb, ub);
  if (ph.nflux != 0) return;
  const double a = ph.half_lambda * wave_speed<D, NC>(ph, uin, uout, n);
  double abar = 0.0;
#pragma unroll
  for (int e = 0; e < NC; ++e) {
    abar = fma(g[e], uin[e] - uout[e], abar);
    ub[e] += side ? -a * g[e] : a * g[e];
  }
  if constexpr (NC > 1) {
    // wave_speed = max(|V_in.n|, |V_out.n|) + max(c_in, c_out); the inner
    // side owns ties (fmax returns its first argument's value)
    const double hb = ph.half_lambda * abar;
    double vn[2] = {0.0, 0.0}, c[2], p[2];
    const double *uu[2] = {uin, uout};
#pragma unroll
    for (int sd = 0; sd < 2; ++sd) {
      double s2 = 0.0;
#pragma unroll
      for (int m = 0; m < D; ++m) {
        s2 += uu[sd][m + 1] * uu[sd][m + 1];
        vn[sd] += (uu[sd][m + 1] / uu[sd][0]) * n[m];
      }
      p[sd] = ph.gm1 * (uu[sd][D + 1] - (0.5 / uu[sd][0]) * s2);
      c[sd] = sqrt(ph.gamma * p[sd] / uu[sd][0]);
    }
    const double ir = 1.0 / us[0];
    if ((fabs(vn[0]) >= fabs(vn[1])) == (side == 0)) {
      // vn = sum_m (m_m / rho) n_m
      const double vb = hb * (vn[side] >= 0.0 ? 1.0 : -1.0);
#pragma unroll
      for (int m = 0; m < D; ++m) ub[m + 1] += vb * n[m] * ir;
      ub[0] -= vb * vn[side] * ir;
    }
    if ((c[0] >= c[1]) == (side == 0)) {
      // c = sqrt(gamma p / rho), p = gm1 (E - |m|^2 / (2 rho))
      const double cs = c[side];
      const double pb = hb * ph.gamma * ir / (2.0 * cs);
      double vv = 0.0;
#pragma unroll
      for (int m = 0; m < D; ++m) {
        const double Vm = us[m + 1] * ir;
        vv = fma(Vm, Vm, vv);
        ub[m + 1] -= pb * ph.gm1 * Vm;
      }
      ub[D + 1] += pb * ph.gm1;
      ub[0] += pb * 0.5 * ph.gm1 * vv - hb * cs * ir * 0.5;
    }
  }
}

template <int D, int NC>
__global__ void __launch_bounds__(256) adj_std_flux_kernel(KernelArgs ka) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const DevGeo &g = ka.geo;
  const Layout &L = ka.layAdjS;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int nq = op.nq, nf = op.nf;
  double *base = smem + (size_t)team * L.team_doubles;
  double *uq = base + L.off[0], *uf = base + L.off[1], *rb = base + L.off[2], *gb = base + L.off[3],
         *fb = base + L.off[4], *t1 = base + L.off[5], *t2 = base + L.off[6], *tf = base + L.off[7];

  for (int t = lane; t < NC * nq; t += tpe) {
    uq[t] = ka.u_q[(size_t)kk * NC * nq + t];
    rb[t] = ka.rbar_q[(size_t)kk * NC * nq + t];
  }
  for (int t = lane; t < NC * nf; t += tpe) {
    uf[t] = ka.u_f[(size_t)kk * NC * nf + t];
    gb[t] = ka.gbar_f[(size_t)kk * NC * nf + t];
  }
  for (int t = lane; t < D * NC * nq; t += tpe) fb[t] = 0.0;
  __syncthreads();
  // r_q += sum_{n,m} D_m^T (hw_mn .* f_n) - hw_mn .* (D_m f_n)
  //   =>  fbar_n += hw_mn .* (D_m rbar_q) - D_m^T (hw_mn .* rbar_q)
  const double *hwl = g.halfWLambda + (size_t)kk * nq * D * D;
  for (int m = 0; m < D; ++m) {
    csr_mul<double, NC>(nq, nq, op.D_ptr[m], op.D_idx[m], op.D_val[m], rb, t1, lane, tpe);
    __syncthreads();
    for (int n = 0; n < D; ++n) {
      const double *hw = hwl + nq * (m + D * n);
      for (int t = lane; t < NC * nq; t += tpe) t2[t] = hw[t % nq] * rb[t];
      __syncthreads();
      double *fn_ = fb + (size_t)n * NC * nq;
      for (int t = lane; t < NC * nq; t += tpe) {
        const int i = t % nq, e = t / nq;
        double acc = 0.0;
        for (int q = op.Dt_ptr[m][i]; q < op.Dt_ptr[m][i + 1]; ++q)
          acc += op.Dt_val[m][q] * t2[e * nq + op.Dt_idx[m][q]];
        fn_[t] += hw[i] * t1[t] - acc;
      }
      __syncthreads();
    }
  }
  // f_f -= halfN_n .* (R f_n)  =>  fbar_n -= R^T (halfN_n .* gbar)
  for (int n = 0; n < D; ++n) {
    for (int t = lane; t < NC * nf; t += tpe) {
      const int j = t % nf;
      tf[t] = 0.5 * g.n_f[n + D * (j + (size_t)nf * kk)] * gb[t];
    }
    __syncthreads();
    double *fn_ = fb + (size_t)n * NC * nq;
    rt_apply<double, NC>(op, op.Rt_val, tf, lane, tpe, [&](int t, double v) { fn_[t] -= v; });
    __syncthreads();
  }
  // f_n = F_n(u_q)  =>  ubar_q = sum_n J_{F_n}^T fbar_n
  for (int i = lane; i < nq; i += tpe) {
    double u[NC], Fb[NC][D], ub[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      u[e] = uq[e * nq + i];
      ub[e] = 0.0;
#pragma unroll
      for (int n = 0; n < D; ++n) Fb[e][n] = fb[(n * NC + e) * nq + i];
    }
    physical_flux_vjp<D, NC>(ph, u, Fb, ub);
    if (live)
#pragma unroll
      for (int e = 0; e < NC; ++e) ka.ubar_q[((size_t)kk * NC + e) * nq + i] = ub[e];
  }
  // interface: own flux w.r.t. the inner state, neighbour's flux w.r.t. its outer state
  for (int j = lane; j < nf; j += tpe) {
    const int P = g.mapP[(size_t)kk * nf + j];
    const int jn = P % nf, kn = P / nf;
    double ui[NC], uo[NC], n[D], nn[D], gown[NC], gnb[NC], ub[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      ui[e] = uf[e * nf + j];
      uo[e] = ka.u_f[((size_t)kn * NC + e) * nf + jn];
      gown[e] = gb[e * nf + j];
      gnb[e] = ka.gbar_f[((size_t)kn * NC + e) * nf + jn];
      ub[e] = 0.0;
    }
#pragma unroll
    for (int m = 0; m < D; ++m) {
      n[m] = g.n_f[m + D * (j + (size_t)nf * kk)];
      nn[m] = g.n_f[m + D * (jn + (size_t)nf * kn)];
    }
    std_iface_bwd<D, NC>(ph, ui, uo, n, gown, 0, ub);
    std_iface_bwd<D, NC>(ph, uo, ui, nn, gnb, 1, ub);
    if (live)
#pragma unroll
      for (int e = 0; e < NC; ++e) ka.ubar_f[((size_t)kk * NC + e) * nf + j] = ub[e];
  }
}

// Transpose of the conservative two-point flux F(uL, uR) = (F(uL) + F(uR))/2
// (advection: a (uL + uR)/2), applied to Fb; adds to ubL and ubR.
template <int D, int NC>
__device__ __forceinline__ void two_point_cons_vjp(const Physics &ph, const double *uL,
                                                   const double *uR, double (&Fb)[NC][D],
                                                   double *ubL, double *ubR) {
#pragma unroll
  for (int e = 0; e < NC; ++e)
#pragma unroll
    for (int n = 0; n < D; ++n) Fb[e][n] *= 0.5;
  physical_flux_vjp<D, NC>(ph, uL, Fb, ubL);
  physical_flux_vjp<D, NC>(ph, uR, Fb, ubR);
}

// FluxDifferencingForm with the conservative two-point flux (scalar
// advection, or Euler with ConservativeFlux): transposes of the volume pairs
// (flux_difference!), the facet-correction pairs (facet_correction!) and
// the interface flux, with the forward's chunked deterministic two-pass
// accumulation -> ubar_q, ubar_f.  Each pair buffer entry holds the
// cotangents of the pair's two states.
template <int D, int NC>
__global__ void __launch_bounds__(256) adj_flux_generic_kernel(KernelArgs ka) {
  extern __shared__ double smem[];
  const DevOps &op = ka.op;
  const Physics &ph = ka.ph;
  const DevGeo &g = ka.geo;
  const Layout &L = ka.layAdjG;
  const int tpe = blockDim.x / ka.epb;
  const int team = threadIdx.x / tpe, lane = threadIdx.x % tpe;
  const int k = blockIdx.x * ka.epb + team;
  const bool live = k < ka.ne;
  const int kk = live ? k : 0;
  const int nq = op.nq, nf = op.nf, nfac = op.nfac, npf = op.npf;
  const float rnpf = qrcp(npf > 0 ? npf : 1);
  double *base = smem + (size_t)team * L.team_doubles;
  double *uq = base + L.off[0], *uf = base + L.off[1], *rb = base + L.off[2], *fb = base + L.off[3],
         *ubq = base + L.off[4], *ubf = base + L.off[5], *Lam = base + L.off[6], *hnq = base + L.off[7],
         *buf = base + L.off[8];
  for (int t = lane; t < NC * nq; t += tpe) {
    uq[t] = ka.u_q[(size_t)kk * NC * nq + t];
    rb[t] = ka.rbar_q[(size_t)kk * NC * nq + t];
    ubq[t] = 0.0;
  }
  for (int t = lane; t < NC * nf; t += tpe) uf[t] = ka.u_f[(size_t)kk * NC * nf + t];
  for (int t = lane; t < nq * D * D; t += tpe) Lam[t] = g.Lambda_q[(size_t)kk * nq * D * D + t];
  if (op.nfp > 0)
    for (int t = lane; t < D * nfac * nq; t += tpe) hnq[t] = g.halfnJq[(size_t)kk * D * nfac * nq + t];
  __syncthreads();
  // fbar_f = -R rbar_q (cotangent of f_f after the BJf scaling)
  csr_mul<double, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_val, rb, fb, lane, tpe);
  __syncthreads();
  for (int t = lane; t < NC * nf; t += tpe) fb[t] = -fb[t];
  // interface: own flux w.r.t. the inner state, neighbour's flux w.r.t. its outer state
  for (int j = lane; j < nf; j += tpe) {
    const int P = g.mapP[(size_t)kk * nf + j];
    const int jn = P % nf, kn = P / nf;
    double ui[NC], uo[NC], n[D], nn[D], gown[NC], gnb[NC], ub[NC];
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
    std_iface_bwd<D, NC>(ph, ui, uo, n, gown, 0, ub);
    std_iface_bwd<D, NC>(ph, uo, ui, nn, gnb, 1, ub);
#pragma unroll
    for (int e = 0; e < NC; ++e) ubf[e * nf + j] = ub[e];
  }
  __syncthreads();

  // volume pairs: diff = sum_m S_m (Lambda_i + Lambda_j)[m, :] . F(u_i, u_j),
  // r_i -= diff, r_j += diff  =>  diffbar = rbar_j - rbar_i
  const int CH = ka.pair_chunk_generic;
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
      double G[D];
#pragma unroll
      for (int n = 0; n < D; ++n) G[n] = 0.0;
#pragma unroll
      for (int m = 0; m < D; ++m) {
        const double Sm = op.vp_S[pidx * D + m];
        if (Sm == 0.0) continue;
#pragma unroll
        for (int n = 0; n < D; ++n)
          G[n] = fma(Sm, Lam[i + nq * (m + D * n)] + Lam[j + nq * (m + D * n)], G[n]);
      }
      double ui[NC], uj[NC], Fb[NC][D];
      double *bi = buf + (size_t)(pidx - c0) * 2 * NC, *bj = bi + NC;
#pragma unroll
      for (int e = 0; e < NC; ++e) {
        ui[e] = uq[e * nq + i];
        uj[e] = uq[e * nq + j];
        const double db = rb[e * nq + j] - rb[e * nq + i];
#pragma unroll
        for (int n = 0; n < D; ++n) Fb[e][n] = db * G[n];
        bi[e] = 0.0;
        bj[e] = 0.0;
      }
      two_point_cons_vjp<D, NC>(ph, ui, uj, Fb, bi, bj);
    }
    __syncthreads();
    // node sums in ascending pair order (inc & 1: the node is the pair's first)
#pragma unroll
    for (int sl = 0; sl < kMaxNodeSlots; ++sl) {
      const int i = lane + sl * tpe;
      if (i >= nq) continue;
      int q = cur[sl];
      const int qe = op.vp_inc_ptr[i + 1];
      for (; q < qe; ++q) {
        const int inc = op.vp_inc[q];
        const int pidx = inc >> 1;
        if (pidx >= c1) break;
        const double *src = buf + (size_t)(pidx - c0) * 2 * NC + ((inc & 1) ? 0 : NC);
#pragma unroll
        for (int e = 0; e < NC; ++e) ubq[e * nq + i] += src[e];
      }
      cur[sl] = q;
    }
    __syncthreads();
  }

  // facet-correction pairs: dp = C_ij nJ . F(u_q[i], u_f[j]), r_i -= dp,
  // f_j -= dp  =>  dpbar = -(rbar_i + fbar_j)
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
        const int f = qdiv(j, rnpf);
        const double Cij = op.fp_C[pidx];
        double nJ[D], ui[NC], uj[NC], Fb[NC][D];
#pragma unroll
        for (int m = 0; m < D; ++m) nJ[m] = Cij * (hnf[m + D * j] + hnq[m + D * (f + nfac * i)]);
        double *bi = buf + (size_t)(pidx - c0) * 2 * NC, *bj = bi + NC;
#pragma unroll
        for (int e = 0; e < NC; ++e) {
          ui[e] = uq[e * nq + i];
          uj[e] = uf[e * nf + j];
          const double db = -(rb[e * nq + i] + fb[e * nf + j]);
#pragma unroll
          for (int m = 0; m < D; ++m) Fb[e][m] = db * nJ[m];
          bi[e] = 0.0;
          bj[e] = 0.0;
        }
        two_point_cons_vjp<D, NC>(ph, ui, uj, Fb, bi, bj);
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
        double *dst = vol ? ubq + r : ubf + r;
        const int stride = vol ? nq : nf;
        int q = cur[sl];
        for (; q < qe; ++q) {
          const int pidx = lst[q];
          if (pidx >= c1) break;
          const double *src = buf + (size_t)(pidx - c0) * 2 * NC + (vol ? 0 : NC);
#pragma unroll
          for (int e = 0; e < NC; ++e) dst[e * stride] += src[e];
        }
        cur[sl] = q;
      }
      __syncthreads();
    }
  }
  if (live) {
    for (int t = lane; t < NC * nq; t += tpe) ka.ubar_q[(size_t)kk * NC * nq + t] = ubq[t];
    for (int t = lane; t < NC * nf; t += tpe) ka.ubar_f[(size_t)kk * NC * nf + t] = ubf[t];
  }
}

// u_q = V u, u_f = R u_q (standard_form_first_order.jl:1-14, and
// flux_differencing_form.jl:253-292 for scalar laws)  =>  mu = V^T (ubar_q + R^T ubar_f)
template <int D, int NC>
__global__ void __launch_bounds__(256) adj_nodal_kernel(KernelArgs ka) {
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
  for (int t = lane; t < NC * nf; t += tpe) F[t] = ka.ubar_f[(size_t)kk * NC * nf + t];
  __syncthreads();
  rt_apply<double, NC>(op, op.Rt_val, F, lane, tpe,
                       [&](int t, double v) { Y[t] = ka.ubar_q[(size_t)kk * NC * nq + t] + v; });
  __syncthreads();
  vdm_tmul<double, D, NC>(op, Y, X, Z, Wb, lane, tpe);
  __syncthreads();
  if (live)
    for (int t = lane; t < NC * np; t += tpe) ka.mu[(size_t)kk * NC * np + t] = X[t];
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
                           Wb, lane, tpe, ka.Akf ? ka.Akf + (size_t)kk * op.np * op.np : nullptr);
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
  const float hl = ph.f_half_lambda, gam = ph.f_gamma;
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
  const float rnpf = qrcp(npf > 0 ? npf : 1);
  const int PS = 4 + D;
  const float gm1 = ph.f_gm1, igm1 = ph.f_igm1;
  const float rho_ref = ph.f_rho_ref, p_ref = ph.f_p_ref;
  const float theta_ref = ph.f_theta_ref, H_ref = ph.f_H_ref;
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
  for (int t = lane; t < nq * D * D; t += tpe) {
    const int v = t / nq, i = t - v * nq;
    Lam[t] = g.Lambda_qn[((size_t)kk * nq + i) * lambda_stride(D) + v];
  }
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
        const int f = qdiv(j, rnpf);
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

// transpose of the mixed-form entropy projection (nodal_values_mixed_kernel):
// the forward recompute uses the same FP32 perturbation maps, and the
// entropy-map Jacobians (symmetric, so the transposes are JVPs) are applied in
// FP32 at the absolute FP32 states
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
  const float *WJf = ka.geo.WJf + (size_t)kk * nq;
  const float *JinvWf = ka.geo.JinvWf + (size_t)kk * nq;
  const float *P1m1 = ka.geo.P1m1f + (size_t)kk * nq, *RP1m1 = ka.geo.RP1m1f + (size_t)kk * nf;

  // ---- forward recompute (as nodal_values_mixed_kernel)
  const double *uk = ka.u + (size_t)kk * NC * np;
  for (int t = lane; t < NC * np; t += tpe) {
    const int e = t / np, l = t - e * np;
    U1[t] = (float)(l == ph.mode0 ? uk[t] - ph.u_ref_modal[e] : uk[t]);
  }
  __syncthreads();
  vdm_mul<float, D, NC>(op, U1, Q0, Zf, Wf, lane, tpe);  // u_q0'
  const EntropyRefF &cr = ph.cref;
  const float gam = ph.f_gamma, gm1 = ph.f_gm1, igm1 = ph.f_igm1;
  const float E_ref = ph.f_E_ref;
  for (int i = lane; i < nq; i += tpe) {
    float ui[NC], wi[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) ui[e] = Q0[e * nq + i];
    cons_to_entropy_pert<D>(cr, ui, wi);
    const float wj = WJf[i];
#pragma unroll
    for (int e = 0; e < NC; ++e) XQ[e * nq + i] = wj * wi[e];
  }
  __syncthreads();
  vdm_tmul<float, D, NC>(op, XQ, T1, Zf, Wf, lane, tpe);
  mass_solve<float, D, NC>(op, JinvWf, nullptr, 1, T1, S1, Zf, Wf, lane, tpe, ka.Akf ? ka.Akf + (size_t)kk * op.np * op.np : nullptr);
  vdm_mul<float, D, NC>(op, T1, WQ, Zf, Wf, lane, tpe);                      // w'_q
  csr_mul<float, NC>(nf, nq, op.R_ptr, op.R_idx, op.R_valf, WQ, WF, lane, tpe);  // w'_f
  __syncthreads();

  // ---- backward: facet then volume entropy-to-conservative transposes
  const float *ubq = reinterpret_cast<const float *>(ka.ubar_q);
  const float *ubf = reinterpret_cast<const float *>(ka.ubar_f);
  for (int t = lane; t < nq + nf; t += tpe) {
    const bool vol = t < nq;
    const int r = vol ? t : t - nq;
    const float p1m1 = vol ? P1m1[r] : RP1m1[r];
    const float *src = vol ? WQ + r : WF + r;
    const int stride = vol ? nq : nf;
    float dwi[NC], wi[NC], bi[NC], ri[NC];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      dwi[e] = fmaf(cr.w_ref[e], p1m1, src[e * stride]);
      wi[e] = cr.w_ref[e] + dwi[e];
      bi[e] = vol ? ubq[(size_t)kk * NC * nq + e * nq + r] : ubf[((size_t)kk * NC + e) * nf + r];
    }
    float alpha, beta, kin;
    entropy_pert_core<D>(cr, dwi, alpha, beta, kin);
    entropy_to_cons_jvp_rhoe_f<D>(gm1, igm1, gam, wi, cr.rhoe_ref * (1.f + beta), bi, ri);
    float *dst = vol ? S1 + r : BF + r;
#pragma unroll
    for (int e = 0; e < NC; ++e) dst[e * stride] = ri[e];
  }
  __syncthreads();
  // wbar_q += R^T wbar_f
  rt_apply<float, NC>(op, op.Rt_valf, BF, lane, tpe, [&](int t, float v) { XQ[t] = S1[t] + v; });
  __syncthreads();
  // projection transpose (V M V^T is symmetric): the same operators
  vdm_tmul<float, D, NC>(op, XQ, T1, Zf, Wf, lane, tpe);
  mass_solve<float, D, NC>(op, JinvWf, nullptr, 1, T1, S1, Zf, Wf, lane, tpe, ka.Akf ? ka.Akf + (size_t)kk * op.np * op.np : nullptr);
  vdm_mul<float, D, NC>(op, T1, XQ, Zf, Wf, lane, tpe);
  // ubar_q0 = J_c2e(u_q0)^T (W J x), symmetric Jacobian
  for (int i = lane; i < nq; i += tpe) {
    float ui[NC], bi[NC], ri[NC];
    const float wj = WJf[i];
#pragma unroll
    for (int e = 0; e < NC; ++e) {
      const float ref = (e == 0) ? cr.rho_ref : ((e == NC - 1) ? E_ref : 0.f);
      ui[e] = ref + Q0[e * nq + i];
      bi[e] = wj * XQ[e * nq + i];
    }
    cons_to_entropy_jvp_f<D>(gam, gm1, igm1, ui, bi, ri);
#pragma unroll
    for (int e = 0; e < NC; ++e) XQ[e * nq + i] = ri[e];
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
  if (!ka.fd) {
#define SSE_STD_ADJ_LIMITS(DD, NN)                                  \
  set((const void *)adj_lift_kernel<DD, NN>, ka.layAdjB1);          \
  set((const void *)adj_std_flux_kernel<DD, NN>, ka.layAdjS);       \
  set((const void *)adj_nodal_kernel<DD, NN>, ka.layAdjB1);
    if (ka.op.d == 2 && ka.op.nc == 1) { SSE_STD_ADJ_LIMITS(2, 1) }
    else if (ka.op.d == 3 && ka.op.nc == 1) { SSE_STD_ADJ_LIMITS(3, 1) }
    else if (ka.op.d == 2 && ka.op.nc == 4) { SSE_STD_ADJ_LIMITS(2, 4) }
    else if (ka.op.d == 3 && ka.op.nc == 5) { SSE_STD_ADJ_LIMITS(3, 5) }
    else return cudaErrorInvalidValue;
#undef SSE_STD_ADJ_LIMITS
    return e;
  }
  if (ka.op.nc == 1 || !ka.ph.ec) {
#define SSE_GEN_ADJ_LIMITS(DD, NN)                                  \
  set((const void *)adj_lift_kernel<DD, NN>, ka.layAdjB1);          \
  set((const void *)adj_flux_generic_kernel<DD, NN>, ka.layAdjG);   \
  set((const void *)adj_nodal_kernel<DD, NN>, ka.layAdjB1);
    if (ka.op.d == 2 && ka.op.nc == 1) { SSE_GEN_ADJ_LIMITS(2, 1) }
    else if (ka.op.d == 3 && ka.op.nc == 1) { SSE_GEN_ADJ_LIMITS(3, 1) }
    else if (ka.op.d == 2 && ka.op.nc == 4) {
      SSE_GEN_ADJ_LIMITS(2, 4)
      set((const void *)adj_projection_kernel<2, 4>, ka.layAdjA);
    } else if (ka.op.d == 3 && ka.op.nc == 5) {
      SSE_GEN_ADJ_LIMITS(3, 5)
      set((const void *)adj_projection_kernel<3, 5>, ka.layAdjA);
    } else return cudaErrorInvalidValue;
#undef SSE_GEN_ADJ_LIMITS
    return e;
  }
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
  if (!ka.fd) {
    const size_t ss = (size_t)ka.epb * ka.layAdjS.team_doubles * sizeof(double);
#define SSE_STD_ADJ_LAUNCH(DD, NN)                                  \
  adj_lift_kernel<DD, NN><<<grid, ka.tpb, s1, st>>>(ka);            \
  adj_std_flux_kernel<DD, NN><<<grid, ka.tpb, ss, st>>>(ka);        \
  adj_nodal_kernel<DD, NN><<<grid, ka.tpb, s1, st>>>(ka);
    if (ka.op.d == 2 && ka.op.nc == 1) { SSE_STD_ADJ_LAUNCH(2, 1) }
    else if (ka.op.d == 3 && ka.op.nc == 1) { SSE_STD_ADJ_LAUNCH(3, 1) }
    else if (ka.op.d == 2 && ka.op.nc == 4) { SSE_STD_ADJ_LAUNCH(2, 4) }
    else if (ka.op.d == 3 && ka.op.nc == 5) { SSE_STD_ADJ_LAUNCH(3, 5) }
    else return cudaErrorInvalidValue;
#undef SSE_STD_ADJ_LAUNCH
    return cudaGetLastError();
  }
  if (ka.op.nc == 1 || !ka.ph.ec) {
    const size_t sg = (size_t)ka.epb * ka.layAdjG.team_doubles * sizeof(double);
    const size_t s3 = (size_t)ka.epb * ka.layAdjA.team_doubles * sizeof(double);
    if (ka.op.d == 2 && ka.op.nc == 1) {
      adj_lift_kernel<2, 1><<<grid, ka.tpb, s1, st>>>(ka);
      adj_flux_generic_kernel<2, 1><<<grid, ka.tpb, sg, st>>>(ka);
      adj_nodal_kernel<2, 1><<<grid, ka.tpb, s1, st>>>(ka);
    } else if (ka.op.d == 3 && ka.op.nc == 1) {
      adj_lift_kernel<3, 1><<<grid, ka.tpb, s1, st>>>(ka);
      adj_flux_generic_kernel<3, 1><<<grid, ka.tpb, sg, st>>>(ka);
      adj_nodal_kernel<3, 1><<<grid, ka.tpb, s1, st>>>(ka);
    } else if (ka.op.d == 2 && ka.op.nc == 4) {
      adj_lift_kernel<2, 4><<<grid, ka.tpb, s1, st>>>(ka);
      adj_flux_generic_kernel<2, 4><<<grid, ka.tpb, sg, st>>>(ka);
      adj_projection_kernel<2, 4><<<grid, ka.tpb, s3, st>>>(ka);
    } else if (ka.op.d == 3 && ka.op.nc == 5) {
      adj_lift_kernel<3, 5><<<grid, ka.tpb, s1, st>>>(ka);
      adj_flux_generic_kernel<3, 5><<<grid, ka.tpb, sg, st>>>(ka);
      adj_projection_kernel<3, 5><<<grid, ka.tpb, s3, st>>>(ka);
    } else {
      return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
  }
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
