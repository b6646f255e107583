/*
 * sse_oracle.c -- CPU restatement (FP64, C99 + OpenMP) of the reference's
 * semi-discrete residual.  TEST INFRASTRUCTURE ONLY: the parity checker for
 * the CUDA library and the timed CPU baseline.  Nothing in the product links
 * or calls it.
 *
 * It consumes exactly the operator/geometry structs of include/sse_gb300.h
 * and follows the reference loop by loop:
 *
 *   semi_discrete_residual! (Threaded)    src/Solvers/Solvers.jl:495-514
 *   nodal_values! (StandardForm)          src/Solvers/standard_form_first_order.jl:1-14
 *   time_derivative! (StandardForm)       src/Solvers/standard_form_first_order.jl:16-63
 *   nodal_values! / entropy_projection!   src/Solvers/flux_differencing_form.jl:190-292
 *   time_derivative! (FD)                 src/Solvers/flux_differencing_form.jl:294-347
 *   flux_difference! (sparse)             src/Solvers/flux_differencing_form.jl:37-75
 *   facet_correction! (sparse)            src/Solvers/flux_differencing_form.jl:126-168
 *   mass_matrix_solve! (WA, Diagonal)     src/Solvers/mass_matrix.jl:177-196
 *   numerical_flux! (LF, central/EC)      src/ConservationLaws/ConservationLaws.jl:75-128
 *   logmean / inv_logmean                 src/ConservationLaws/ConservationLaws.jl:132-156
 *   Euler fluxes, entropy variables       src/ConservationLaws/euler_navierstokes.jl:58-225
 *   advection fluxes                      src/ConservationLaws/linear_advection_diffusion.jl:54-128
 *   WarpedTensorProductMap mul!/transpose src/MatrixFreeOperators/warped_product_2d.jl:31-89,
 *                                         src/MatrixFreeOperators/warped_product_3d.jl:47-136
 *   conservation residuals                src/Analysis/conservation.jl:145-189
 *
 * Time stepping restates OrdinaryDiffEq's fixed-step CarpenterKennedy2N54
 * (Carpenter & Kennedy 1994, NASA TM-109112, 5-stage 4th-order 2N-storage
 * scheme) and classic RK4 as the reference's tests call them
 * (test/test_driver.jl:78-84).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/sse_gb300.h"

#define MAXC 5
#define MAXD 3

/* Scalar type of every state-dependent quantity: double here.  The tangent
 * build (sse_oracle_tangent.cpp) compiles this same file as C++ with a
 * dual-number type, so its derivatives are those of exactly this
 * restatement.  Operator and geometry values stay double. */
#ifndef SSE_ORACLE_REAL
#define SSE_ORACLE_REAL double
#endif
typedef SSE_ORACLE_REAL sse_real;

typedef struct {
  sse_config cfg;
  sse_operators ops;
  sse_geometry geo;
  sse_real *u_q; /* N_q x N_c x N_e */
  sse_real *u_f; /* N_f x N_e x N_c */
  int nthreads;
} oracle_t;

/* ------------------------------------------------------------------ */
/* sparse and warped tensor-product maps                               */
/* ------------------------------------------------------------------ */

/* y = A x (CSC), y zeroed first */
static void csc_mul(const sse_csc *A, const sse_real *x, sse_real *y) {
  for (int64_t i = 0; i < A->m; ++i) y[i] = 0.0;
  for (int64_t j = 0; j < A->n; ++j) {
    sse_real xj = x[j];
    for (int64_t ii = A->colptr[j] - 1; ii < A->colptr[j + 1] - 1; ++ii)
      y[A->rowval[ii] - 1] += A->nzval[ii] * xj;
  }
}

/* y = A^T x (CSC) */
static void csc_tmul(const sse_csc *A, const sse_real *x, sse_real *y) {
  for (int64_t j = 0; j < A->n; ++j) {
    sse_real acc = 0.0;
    for (int64_t ii = A->colptr[j] - 1; ii < A->colptr[j + 1] - 1; ++ii)
      acc += A->nzval[ii] * x[A->rowval[ii] - 1];
    y[j] = acc;
  }
}

/* V x for the warped tensor-product Vandermonde; x has N_p entries, y N_q.
 * warped_product_2d.jl:31-55, warped_product_3d.jl:47-84 */
static void vdm_mul(const oracle_t *o, const sse_real *x, sse_real *y) {
  const sse_operators *op = &o->ops;
  if (op->V_dense) {
    /* dense V of a multidimensional basis (multidimensional.jl:1-41) */
    const int nq = o->cfg.n_q, np = o->cfg.n_p;
    for (int i = 0; i < nq; ++i) {
      sse_real t = 0.0;
      for (int a = 0; a < np; ++a) t = fma(op->V_dense[i + (size_t)nq * a], x[a], t);
      y[i] = t;
    }
    return;
  }
  if (!op->vdm_A) { memcpy(y, x, sizeof(sse_real) * o->cfg.n_q); return; }
  const int p1 = op->vdm_p + 1;
  const int M1 = op->vdm_m[0], M2 = op->vdm_m[1], M3 = op->vdm_m[2];
  if (o->cfg.d == 2) {
    sse_real Z[16 * 16];
    for (int a2 = 0; a2 < M2; ++a2)
      for (int b1 = 0; b1 < p1; ++b1) {
        sse_real t = 0.0;
        for (int b2 = 0; b2 < p1 - b1; ++b2) {
          int64_t l = op->vdm_sigma_in[b1 + p1 * b2] - 1;
          t = fma(op->vdm_B[a2 + M2 * (b1 + p1 * b2)], x[l], t);
        }
        Z[b1 + p1 * a2] = t;
      }
    for (int a1 = 0; a1 < M1; ++a1)
      for (int a2 = 0; a2 < M2; ++a2) {
        sse_real t = 0.0;
        for (int b1 = 0; b1 < p1; ++b1) t = fma(op->vdm_A[a1 + M1 * b1], Z[b1 + p1 * a2], t);
        y[M2 * a1 + a2] = t;
      }
    return;
  }
  sse_real Z[8 * 8 * 8], W[8 * 8 * 8];
  for (int b1 = 0; b1 < p1; ++b1)
    for (int b2 = 0; b2 < p1 - b1; ++b2)
      for (int a3 = 0; a3 < M3; ++a3) {
        sse_real t = 0.0;
        for (int b3 = 0; b3 < p1 - b1 - b2; ++b3) {
          int64_t l = op->vdm_sigma_in[b1 + p1 * (b2 + p1 * b3)] - 1;
          t = fma(op->vdm_C[a3 + M3 * (b1 + p1 * (b2 + p1 * b3))], x[l], t);
        }
        Z[b1 + p1 * (b2 + p1 * a3)] = t;
      }
  for (int b1 = 0; b1 < p1; ++b1)
    for (int a2 = 0; a2 < M2; ++a2)
      for (int a3 = 0; a3 < M3; ++a3) {
        sse_real t = 0.0;
        for (int b2 = 0; b2 < p1 - b1; ++b2)
          t = fma(op->vdm_B[a2 + M2 * (b1 + p1 * b2)], Z[b1 + p1 * (b2 + p1 * a3)], t);
        W[b1 + p1 * (a2 + M2 * a3)] = t;
      }
  for (int a1 = 0; a1 < M1; ++a1)
    for (int a2 = 0; a2 < M2; ++a2)
      for (int a3 = 0; a3 < M3; ++a3) {
        sse_real t = 0.0;
        for (int b1 = 0; b1 < p1; ++b1) t = fma(op->vdm_A[a1 + M1 * b1], W[b1 + p1 * (a2 + M2 * a3)], t);
        y[M2 * M3 * a1 + M3 * a2 + a3] = t;
      }
}

/* V^T x; warped_product_2d.jl:61-89, warped_product_3d.jl:94-136 */
static void vdm_tmul(const oracle_t *o, const sse_real *x, sse_real *y) {
  const sse_operators *op = &o->ops;
  if (op->V_dense) {
    const int nq = o->cfg.n_q, np = o->cfg.n_p;
    for (int a = 0; a < np; ++a) {
      sse_real t = 0.0;
      for (int i = 0; i < nq; ++i) t = fma(op->V_dense[i + (size_t)nq * a], x[i], t);
      y[a] = t;
    }
    return;
  }
  if (!op->vdm_A) { memcpy(y, x, sizeof(sse_real) * o->cfg.n_q); return; }
  const int p1 = op->vdm_p + 1;
  const int M1 = op->vdm_m[0], M2 = op->vdm_m[1], M3 = op->vdm_m[2];
  if (o->cfg.d == 2) {
    sse_real Z[16 * 16];
    for (int b1 = 0; b1 < p1; ++b1)
      for (int a2 = 0; a2 < M2; ++a2) {
        sse_real t = 0.0;
        for (int a1 = 0; a1 < M1; ++a1) t = fma(op->vdm_A[a1 + M1 * b1], x[M2 * a1 + a2], t);
        Z[b1 + p1 * a2] = t;
      }
    for (int b1 = 0; b1 < p1; ++b1)
      for (int b2 = 0; b2 < p1 - b1; ++b2) {
        sse_real t = 0.0;
        for (int a2 = 0; a2 < M2; ++a2) t = fma(op->vdm_B[a2 + M2 * (b1 + p1 * b2)], Z[b1 + p1 * a2], t);
        y[op->vdm_sigma_in[b1 + p1 * b2] - 1] = t;
      }
    return;
  }
  sse_real Z[8 * 8 * 8], W[8 * 8 * 8];
  for (int b1 = 0; b1 < p1; ++b1)
    for (int a2 = 0; a2 < M2; ++a2)
      for (int a3 = 0; a3 < M3; ++a3) {
        sse_real t = 0.0;
        for (int a1 = 0; a1 < M1; ++a1)
          t = fma(op->vdm_A[a1 + M1 * b1], x[M2 * M3 * a1 + M3 * a2 + a3], t);
        W[b1 + p1 * (a2 + M2 * a3)] = t;
      }
  for (int b1 = 0; b1 < p1; ++b1)
    for (int b2 = 0; b2 < p1 - b1; ++b2)
      for (int a3 = 0; a3 < M3; ++a3) {
        sse_real t = 0.0;
        for (int a2 = 0; a2 < M2; ++a2)
          t = fma(op->vdm_B[a2 + M2 * (b1 + p1 * b2)], W[b1 + p1 * (a2 + M2 * a3)], t);
        Z[b1 + p1 * (b2 + p1 * a3)] = t;
      }
  for (int b1 = 0; b1 < p1; ++b1)
    for (int b2 = 0; b2 < p1 - b1; ++b2)
      for (int b3 = 0; b3 < p1 - b1 - b2; ++b3) {
        sse_real t = 0.0;
        for (int a3 = 0; a3 < M3; ++a3)
          t = fma(op->vdm_C[a3 + M3 * (b1 + p1 * (b2 + p1 * b3))], Z[b1 + p1 * (b2 + p1 * a3)], t);
        y[op->vdm_sigma_in[b1 + p1 * (b2 + p1 * b3)] - 1] = t;
      }
}

/* ------------------------------------------------------------------ */
/* physics                                                             */
/* ------------------------------------------------------------------ */

/* ConservationLaws.jl:132-145 */
static sse_real logmean(sse_real x, sse_real y) {
  sse_real f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4) return (x + y) * 105 / (210 + f2 * (70 + f2 * (42 + f2 * 30)));
  return (y - x) / log(y / x);
}

/* ConservationLaws.jl:147-156 */
static sse_real inv_logmean(sse_real x, sse_real y) {
  sse_real f2 = (x * (x - 2 * y) + y * y) / (x * (x + 2 * y) + y * y);
  if (f2 < 1.0e-4) return (210 + f2 * (70 + f2 * (42 + f2 * 30))) / ((x + y) * 105);
  return log(y / x) / (y - x);
}

/* two-point flux tensor F[e + MAXC*n] (e = 0..N_c-1, n = 0..d-1); kind 1:
 * Euler EC, euler_navierstokes.jl:171-195 (Ranocha); kind 2: Chandrashekar
 * (2013), an option with no reference counterpart; kind 0: conservative
 * average, :152-158; advection: linear_advection_diffusion.jl:113-119. */
static void two_point_flux(const sse_config *c, int kind, const sse_real *uL, const sse_real *uR,
                           sse_real *F) {
  const int ec = kind == 1;
  const int d = c->d;
  if (c->law == SSE_LINEAR_ADVECTION) {
    sse_real f1 = 0.5 * (uL[0] + uR[0]);
    for (int m = 0; m < d; ++m) F[MAXC * m] = c->a[m] * f1;
    return;
  }
  const double gm1 = c->gamma - 1.0, igm1 = 1.0 / (c->gamma - 1.0);
  const int E = d + 1;
  if (ec) {
    sse_real VL[MAXD], VR[MAXD], sL = 0.0, sR = 0.0, vv = 0.0;
    for (int m = 0; m < d; ++m) { VL[m] = uL[m + 1] / uL[0]; VR[m] = uR[m + 1] / uR[0]; }
    for (int m = 0; m < d; ++m) { sL += VL[m] * VL[m]; sR += VR[m] * VR[m]; }
    sse_real pL = gm1 * (uL[E] - 0.5 * uL[0] * sL);
    sse_real pR = gm1 * (uR[E] - 0.5 * uR[0] * sR);
    sse_real rho_avg = logmean(uL[0], uR[0]);
    sse_real Vavg[MAXD];
    for (int m = 0; m < d; ++m) Vavg[m] = 0.5 * (VL[m] + VR[m]);
    sse_real pavg = 0.5 * (pL + pR);
    for (int m = 0; m < d; ++m) vv += VL[m] * VR[m];
    sse_real C = 0.5 * vv + igm1 * inv_logmean(uL[0] / pL, uR[0] / pR);
    for (int n = 0; n < d; ++n) {
      sse_real frho = rho_avg * Vavg[n];
      F[0 + MAXC * n] = frho;
      for (int m = 0; m < d; ++m)
        F[m + 1 + MAXC * n] = rho_avg * Vavg[m] * Vavg[n] + (m == n ? pavg : 0.0);
      F[E + MAXC * n] = frho * C + 0.5 * (pL * VR[n] + pR * VL[n]);
    }
    return;
  }
  if (kind == 2) {
    /* Chandrashekar: rho_hat, beta_hat logarithmic means, beta = rho / (2 p),
     * p_hat = avg(rho) / (2 avg(beta)) */
    sse_real VL[MAXD], VR[MAXD], sL = 0.0, sR = 0.0, Vb[MAXD];
    for (int m = 0; m < d; ++m) {
      VL[m] = uL[m + 1] / uL[0];
      VR[m] = uR[m + 1] / uR[0];
      sL += VL[m] * VL[m];
      sR += VR[m] * VR[m];
      Vb[m] = 0.5 * (VL[m] + VR[m]);
    }
    sse_real pL = gm1 * (uL[E] - 0.5 * uL[0] * sL);
    sse_real pR = gm1 * (uR[E] - 0.5 * uR[0] * sR);
    sse_real bL = uL[0] / (2.0 * pL), bR = uR[0] / (2.0 * pR);
    sse_real rho_hat = logmean(uL[0], uR[0]), beta_hat = logmean(bL, bR);
    sse_real p_hat = 0.5 * (uL[0] + uR[0]) / (bL + bR);
    sse_real h = 1.0 / (2.0 * gm1 * beta_hat) - 0.25 * (sL + sR);
    for (int n = 0; n < d; ++n) {
      sse_real frho = rho_hat * Vb[n], fe = frho * h;
      F[0 + MAXC * n] = frho;
      for (int m = 0; m < d; ++m) {
        sse_real fm = frho * Vb[m] + (m == n ? p_hat : 0.0);
        F[m + 1 + MAXC * n] = fm;
        fe += fm * Vb[m];
      }
      F[E + MAXC * n] = fe;
    }
    return;
  }
  /* ConservativeFlux: average of physical fluxes (euler_navierstokes.jl:58-68) */
  const sse_real *us[2] = {uL, uR};
  for (int n = 0; n < d; ++n)
    for (int e = 0; e < d + 2; ++e) F[e + MAXC * n] = 0.0;
  for (int s = 0; s < 2; ++s) {
    const sse_real *u = us[s];
    sse_real V[MAXD], sum = 0.0;
    for (int m = 0; m < d; ++m) V[m] = u[m + 1] / u[0];
    for (int m = 0; m < d; ++m) sum += u[m + 1] * V[m];
    sse_real p = gm1 * (u[E] - 0.5 * sum);
    sse_real ht = u[E] + p;
    for (int n = 0; n < d; ++n) {
      F[0 + MAXC * n] += u[n + 1];
      for (int m = 0; m < d; ++m) F[m + 1 + MAXC * n] += u[m + 1] * V[n] + (m == n ? p : 0.0);
      F[E + MAXC * n] += ht * V[n];
    }
  }
  for (int n = 0; n < d; ++n)
    for (int e = 0; e < d + 2; ++e) F[e + MAXC * n] *= 0.5;
}

/* physical flux f[e + MAXC*n] (euler_navierstokes.jl:58-68; advection :54-61) */
static void physical_flux(const sse_config *c, const sse_real *u, sse_real *F) {
  const int d = c->d;
  if (c->law == SSE_LINEAR_ADVECTION) {
    for (int m = 0; m < d; ++m) F[MAXC * m] = c->a[m] * u[0];
    return;
  }
  const double gm1 = c->gamma - 1.0;
  const int E = d + 1;
  sse_real V[MAXD], sum = 0.0;
  for (int m = 0; m < d; ++m) V[m] = u[m + 1] / u[0];
  for (int m = 0; m < d; ++m) sum += u[m + 1] * V[m];
  sse_real p = gm1 * (u[E] - 0.5 * sum);
  sse_real ht = u[E] + p;
  for (int n = 0; n < d; ++n) {
    F[0 + MAXC * n] = u[n + 1];
    for (int m = 0; m < d; ++m) F[m + 1 + MAXC * n] = u[m + 1] * V[n] + (m == n ? p : 0.0);
    F[E + MAXC * n] = ht * V[n];
  }
}

/* euler_navierstokes.jl:133-150; linear_advection_diffusion.jl:106-111 */
static sse_real wave_speed(const sse_config *c, const sse_real *ui, const sse_real *uo, const double *n) {
  const int d = c->d;
  if (c->law == SSE_LINEAR_ADVECTION) {
    double s = 0.0;
    for (int m = 0; m < d; ++m) s += c->a[m] * n[m];
    return fabs(s);
  }
  const double gm1 = c->gamma - 1.0;
  const int E = d + 1;
  sse_real si = 0.0, so = 0.0, vni = 0.0, vno = 0.0;
  for (int m = 0; m < d; ++m) { si += ui[m + 1] * ui[m + 1]; so += uo[m + 1] * uo[m + 1]; }
  sse_real pi_ = gm1 * (ui[E] - (0.5 / ui[0]) * si);
  sse_real po = gm1 * (uo[E] - (0.5 / uo[0]) * so);
  for (int m = 0; m < d; ++m) { vni += (ui[m + 1] / ui[0]) * n[m]; vno += (uo[m + 1] / uo[0]) * n[m]; }
  sse_real ci = sqrt(c->gamma * pi_ / ui[0]);
  sse_real co = sqrt(c->gamma * po / uo[0]);
  return fmax(fabs(vni), fabs(vno)) + fmax(ci, co);
}

/* euler_navierstokes.jl:100-113 */
static void cons_to_entropy(const sse_config *c, const sse_real *u, sse_real *w) {
  const int d = c->d, E = d + 1;
  const double g = c->gamma, gm1 = g - 1.0, igm1 = 1.0 / (g - 1.0);
  sse_real s = 0.0;
  for (int m = 0; m < d; ++m) s += u[m + 1] * u[m + 1];
  sse_real k = (0.5 / u[0]) * s;
  sse_real p = gm1 * (u[E] - k);
  sse_real ip = 1.0 / p;
  w[0] = igm1 * (g - log(p / pow(u[0], g))) - k * ip;
  for (int m = 0; m < d; ++m) w[m + 1] = u[m + 1] * ip;
  w[E] = -u[0] * ip;
}

/* euler_navierstokes.jl:115-131 */
static void entropy_to_cons(const sse_config *c, const sse_real *w_in, sse_real *u) {
  const int d = c->d, E = d + 1;
  const double g = c->gamma, gm1 = g - 1.0, igm1 = 1.0 / (g - 1.0);
  sse_real w[MAXC];
  for (int e = 0; e < d + 2; ++e) w[e] = w_in[e] * gm1;
  sse_real s = 0.0;
  for (int m = 0; m < d; ++m) s += w[m + 1] * w[m + 1];
  sse_real k = s / (2 * w[E]);
  sse_real sv = g - w[0] + k;
  sse_real rhoe = pow(gm1 / pow(-w[E], g), igm1) * exp(-sv * igm1);
  u[0] = -w[E] * rhoe;
  for (int m = 0; m < d; ++m) u[m + 1] = w[m + 1] * rhoe;
  u[E] = rhoe * (1 - k);
}

/* numerical_flux! (ConservationLaws.jl:75-128) at facet node i: fstar[e] */
static void numerical_flux(const sse_config *c, int two_point_ec, const sse_real *ui,
                           const sse_real *uo, const double *n, sse_real *fstar) {
  sse_real F[MAXC * MAXD];
  two_point_flux(c, two_point_ec, ui, uo, F);
  sse_real a = 0.0;
  if (c->numerical_flux == SSE_LAX_FRIEDRICHS) a = c->half_lambda * wave_speed(c, ui, uo, n);
  for (int e = 0; e < c->n_c; ++e) {
    sse_real fn = 0.0;
    for (int m = 0; m < c->d; ++m) fn = fma(F[e + MAXC * m], n[m], fn);
    fstar[e] = (c->numerical_flux == SSE_LAX_FRIEDRICHS) ? fma(a, ui[e] - uo[e], fn) : fn;
  }
}

/* ------------------------------------------------------------------ */
/* per-element phases                                                  */
/* ------------------------------------------------------------------ */

typedef struct {
  sse_real *a, *b, *c, *w, *fq, *ff, *fn, *rq;
} scratch_t;

static size_t scratch_len(const sse_config *c) {
  size_t nq = c->n_q, nf = c->n_f, nc = c->n_c, np = c->n_p, d = c->d;
  size_t big = nq > nf ? nq : nf;
  if (np > big) big = np;
  return 4 * big * nc + nq * nc * d + 3 * nf * nc + nq * nc + 64;
}

static void scratch_carve(const sse_config *c, sse_real *base, scratch_t *s) {
  size_t nq = c->n_q, nf = c->n_f, nc = c->n_c, np = c->n_p, d = c->d;
  size_t big = nq > nf ? nq : nf;
  if (np > big) big = np;
  s->a = base; base += big * nc;
  s->b = base; base += big * nc;
  s->c = base; base += big * nc;
  s->w = base; base += big * nc;
  s->fq = base; base += nq * nc * d;
  s->ff = base; base += nf * nc;
  s->fn = base; base += nf * nc;
  s->rq = base; base += nq * nc;
}

/* WeightAdjustedSolver (M^-1 = I) / DiagonalSolver solve on one element,
 * rhs (N_p x N_c) in place; mass_matrix.jl:177-196 */
static void mass_solve(const oracle_t *o, int k, sse_real *rhs, sse_real *tmp) {
  const sse_config *c = &o->cfg;
  const int nq = c->n_q, np = c->n_p;
  if (c->mass_solver == SSE_DIAGONAL) {
    const double *wji = o->geo.WJinv + (size_t)nq * k;
    for (int e = 0; e < c->n_c; ++e)
      for (int i = 0; i < np; ++i) rhs[i + np * e] *= wji[i];
    return;
  }
  const double *jw = o->geo.JinvW + (size_t)nq * k;
  for (int e = 0; e < c->n_c; ++e) {
    vdm_mul(o, rhs + np * e, tmp);
    for (int i = 0; i < nq; ++i) tmp[i] *= jw[i];
    vdm_tmul(o, tmp, rhs + np * e);
  }
}

static void nodal_values_elem(oracle_t *o, const sse_real *u, int k, scratch_t *s) {
  const sse_config *c = &o->cfg;
  const int nq = c->n_q, nf = c->n_f, nc = c->n_c, np = c->n_p, ne = c->n_e;
  const sse_real *uk = u + (size_t)np * nc * k;
  sse_real *uq = o->u_q + (size_t)nq * nc * k;
  const int project = (c->form == SSE_FLUX_DIFFERENCING_FORM && c->law == SSE_EULER);
  if (!project) {
    /* u_q = V u; u_f = R u_q */
    for (int e = 0; e < nc; ++e) {
      vdm_mul(o, uk + np * e, uq + nq * e);
      csc_mul(&o->ops.R, uq + nq * e, s->a);
      for (int j = 0; j < nf; ++j) o->u_f[j + (size_t)nf * k + (size_t)nf * ne * e] = s->a[j];
    }
    return;
  }
  sse_real ui[MAXC], wi[MAXC];
  if (!o->ops.vdm_A && !o->ops.V_dense) {
    /* nodal entropy projection (flux_differencing_form.jl:190-211) */
    for (int e = 0; e < nc; ++e) memcpy(uq + nq * e, uk + np * e, sizeof(sse_real) * nq);
    sse_real *wq = s->a, *wf = s->b;
    for (int i = 0; i < nq; ++i) {
      for (int e = 0; e < nc; ++e) ui[e] = uq[i + nq * e];
      cons_to_entropy(c, ui, wi);
      for (int e = 0; e < nc; ++e) wq[i + nq * e] = wi[e];
    }
    for (int e = 0; e < nc; ++e) csc_mul(&o->ops.R, wq + nq * e, wf + nf * e);
    for (int j = 0; j < nf; ++j) {
      for (int e = 0; e < nc; ++e) wi[e] = wf[j + nf * e];
      entropy_to_cons(c, wi, ui);
      for (int e = 0; e < nc; ++e) o->u_f[j + (size_t)nf * k + (size_t)nf * ne * e] = ui[e];
    }
    return;
  }
  /* modal entropy projection (flux_differencing_form.jl:214-250) */
  sse_real *wq = s->a, *wf = s->b, *w = s->c, *tmp = s->w;
  const double *WJ = o->geo.WJ + (size_t)nq * k;
  for (int e = 0; e < nc; ++e) vdm_mul(o, uk + np * e, uq + nq * e);
  for (int i = 0; i < nq; ++i) {
    for (int e = 0; e < nc; ++e) ui[e] = uq[i + nq * e];
    cons_to_entropy(c, ui, wi);
    for (int e = 0; e < nc; ++e) wq[i + nq * e] = wi[e];
  }
  for (int e = 0; e < nc; ++e) {
    for (int i = 0; i < nq; ++i) wq[i + nq * e] *= WJ[i];
    vdm_tmul(o, wq + nq * e, w + np * e);
  }
  mass_solve(o, k, w, tmp);
  for (int e = 0; e < nc; ++e) {
    vdm_mul(o, w + np * e, wq + nq * e);
    csc_mul(&o->ops.R, wq + nq * e, wf + nf * e);
  }
  for (int i = 0; i < nq; ++i) {
    for (int e = 0; e < nc; ++e) wi[e] = wq[i + nq * e];
    entropy_to_cons(c, wi, ui);
    for (int e = 0; e < nc; ++e) uq[i + nq * e] = ui[e];
  }
  for (int j = 0; j < nf; ++j) {
    for (int e = 0; e < nc; ++e) wi[e] = wf[j + nf * e];
    entropy_to_cons(c, wi, ui);
    for (int e = 0; e < nc; ++e) o->u_f[j + (size_t)nf * k + (size_t)nf * ne * e] = ui[e];
  }
}

static void numerical_flux_elem(oracle_t *o, int k, int two_point_ec, sse_real *ff) {
  const sse_config *c = &o->cfg;
  const int nf = c->n_f, nc = c->n_c, ne = c->n_e, d = c->d;
  sse_real ui[MAXC], uo[MAXC], fs[MAXC];
  double nn[MAXD];
  for (int i = 0; i < nf; ++i) {
    int64_t P = o->geo.mapP[i + (size_t)nf * k] - 1;
    for (int e = 0; e < nc; ++e) {
      ui[e] = o->u_f[i + (size_t)nf * k + (size_t)nf * ne * e];
      uo[e] = o->u_f[P + (size_t)nf * ne * e];
    }
    for (int m = 0; m < d; ++m) nn[m] = o->geo.n_f[m + d * (i + (size_t)nf * k)];
    numerical_flux(c, two_point_ec, ui, uo, nn, fs);
    for (int e = 0; e < nc; ++e) ff[i + nf * e] = fs[e];
  }
}

/* StandardForm, ReferenceOperators: standard_form_first_order.jl:16-63 */
static void time_derivative_standard(oracle_t *o, sse_real *dudt, int k, scratch_t *s) {
  const sse_config *c = &o->cfg;
  const int nq = c->n_q, nf = c->n_f, nc = c->n_c, np = c->n_p, d = c->d;
  sse_real *uq = o->u_q + (size_t)nq * nc * k;
  sse_real F[MAXC * MAXD], ui[MAXC];
  /* f_q[i, e, n] */
  for (int i = 0; i < nq; ++i) {
    for (int e = 0; e < nc; ++e) ui[e] = uq[i + nq * e];
    physical_flux(c, ui, F);
    for (int n = 0; n < d; ++n)
      for (int e = 0; e < nc; ++e) s->fq[i + nq * (e + nc * n)] = F[e + MAXC * n];
  }
  numerical_flux_elem(o, k, 0, s->ff);
  for (int x = 0; x < nq * nc; ++x) s->rq[x] = 0.0;
  for (int n = 0; n < d; ++n) {
    for (int m = 0; m < d; ++m) {
      const double *hw = o->geo.halfWLambda + (size_t)nq * (m + d * (n + d * (size_t)k));
      for (int e = 0; e < nc; ++e) {
        const sse_real *fqn = s->fq + nq * (e + nc * n);
        for (int i = 0; i < nq; ++i) s->a[i] = hw[i] * fqn[i];
        csc_tmul(&o->ops.D[m], s->a, s->b);
        for (int i = 0; i < nq; ++i) s->rq[i + nq * e] += s->b[i];
        csc_mul(&o->ops.D[m], fqn, s->b);
        for (int i = 0; i < nq; ++i) s->b[i] *= hw[i];
        for (int i = 0; i < nq; ++i) s->rq[i + nq * e] -= s->b[i];
      }
    }
    for (int e = 0; e < nc; ++e) {
      csc_mul(&o->ops.R, s->fq + nq * (e + nc * n), s->fn + nf * e);
      for (int j = 0; j < nf; ++j) {
        double halfN = 0.5 * o->geo.n_f[n + d * (j + (size_t)nf * k)];
        s->ff[j + nf * e] -= s->fn[j + nf * e] * halfN;
      }
    }
  }
  const double *bjf = o->geo.BJf + (size_t)nf * k;
  for (int e = 0; e < nc; ++e) {
    for (int j = 0; j < nf; ++j) s->ff[j + nf * e] *= bjf[j];
    csc_tmul(&o->ops.R, s->ff + nf * e, s->a);
    for (int i = 0; i < nq; ++i) s->rq[i + nq * e] -= s->a[i];
  }
  sse_real *dk = dudt + (size_t)np * nc * k;
  for (int e = 0; e < nc; ++e) vdm_tmul(o, s->rq + nq * e, dk + np * e);
  mass_solve(o, k, dk, s->a);
}

/* FluxDifferencingForm: flux_differencing_form.jl:294-347 */
static void time_derivative_fd(oracle_t *o, sse_real *dudt, int k, scratch_t *s) {
  const sse_config *c = &o->cfg;
  const int nq = c->n_q, nf = c->n_f, nc = c->n_c, np = c->n_p, d = c->d, ne = c->n_e;
  const int ec = (c->two_point_flux == SSE_EC_FLUX) ? 1 : (c->two_point_flux == SSE_CHANDRASHEKAR_FLUX ? 2 : 0);
  sse_real *uq = o->u_q + (size_t)nq * nc * k;
  sse_real F[MAXC * MAXD], ui[MAXC], uj[MAXC];
  numerical_flux_elem(o, k, ec, s->ff);
  const double *bjf = o->geo.BJf + (size_t)nf * k;
  for (int e = 0; e < nc; ++e)
    for (int j = 0; j < nf; ++j) s->ff[j + nf * e] *= bjf[j];
  /* flux_difference! (sparse), :37-75 */
  const double *Lq = o->geo.Lambda_q + (size_t)nq * d * d * k;
  for (int x = 0; x < nq * nc; ++x) s->rq[x] = 0.0;
  for (int m = 0; m < d; ++m) {
    const sse_csc *S = &o->ops.S[m];
    for (int64_t j = 0; j < S->n; ++j) {
      for (int64_t ii = S->colptr[j] - 1; ii < S->colptr[j + 1] - 1; ++ii) {
        int64_t i = S->rowval[ii] - 1;
        if (i < j) {
          for (int e = 0; e < nc; ++e) { ui[e] = uq[i + nq * e]; uj[e] = uq[j + nq * e]; }
          two_point_flux(c, ec, ui, uj, F);
          double Sij = S->nzval[ii];
          for (int e = 0; e < nc; ++e) {
            sse_real Fm = 0.0;
            for (int n = 0; n < d; ++n) {
              double Lij = Lq[i + nq * (m + d * n)] + Lq[j + nq * (m + d * n)];
              Fm = fma(Lij, F[e + MAXC * n], Fm);
            }
            sse_real diff = Sij * Fm;
            s->rq[i + nq * e] -= diff;
            s->rq[j + nq * e] += diff;
          }
        }
      }
    }
  }
  /* facet_correction! (sparse), :126-168 */
  const sse_csc *C = &o->ops.C;
  if (C->colptr && C->n > 0) {
    const double *hnf = o->geo.halfnJf + (size_t)d * nf * k;
    const double *hnq = o->geo.halfnJq + (size_t)d * c->num_faces * nq * k;
    for (int64_t j = 0; j < C->n; ++j) {
      int f = (int)(j / c->nodes_per_face);
      for (int e = 0; e < nc; ++e) uj[e] = o->u_f[j + (size_t)nf * k + (size_t)nf * ne * e];
      for (int64_t ii = C->colptr[j] - 1; ii < C->colptr[j + 1] - 1; ++ii) {
        int64_t i = C->rowval[ii] - 1;
        for (int e = 0; e < nc; ++e) ui[e] = uq[i + nq * e];
        two_point_flux(c, ec, ui, uj, F);
        double Cij = C->nzval[ii];
        for (int e = 0; e < nc; ++e) {
          sse_real Fn = 0.0;
          for (int m = 0; m < d; ++m) {
            double nJ = hnf[m + d * j] + hnq[m + d * (f + c->num_faces * i)];
            Fn = fma(nJ, F[e + MAXC * m], Fn);
          }
          sse_real diff = Cij * Fn;
          s->rq[i + nq * e] -= diff;
          s->ff[j + nf * e] -= diff;
        }
      }
    }
  }
  for (int e = 0; e < nc; ++e) {
    csc_tmul(&o->ops.R, s->ff + nf * e, s->a);
    for (int i = 0; i < nq; ++i) s->rq[i + nq * e] -= s->a[i];
  }
  sse_real *dk = dudt + (size_t)np * nc * k;
  for (int e = 0; e < nc; ++e) vdm_tmul(o, s->rq + nq * e, dk + np * e);
  mass_solve(o, k, dk, s->a);
}

/* ------------------------------------------------------------------ */
/* public entry points (test infrastructure)                           */
/* ------------------------------------------------------------------ */

void *oracle_create(const sse_config *cfg, const sse_operators *ops, const sse_geometry *geo,
                    int nthreads) {
  oracle_t *o = (oracle_t *)calloc(1, sizeof(oracle_t));
  o->cfg = *cfg;
  o->ops = *ops;
  o->geo = *geo;
  o->u_q = (sse_real *)malloc(sizeof(sse_real) * (size_t)cfg->n_q * cfg->n_c * cfg->n_e);
  o->u_f = (sse_real *)malloc(sizeof(sse_real) * (size_t)cfg->n_f * cfg->n_c * cfg->n_e);
  o->nthreads = nthreads > 0 ? nthreads : 1;
  return o;
}

void oracle_destroy(void *h) {
  oracle_t *o = (oracle_t *)h;
  if (!o) return;
  free(o->u_q);
  free(o->u_f);
  free(o);
}

int oracle_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static void run_nodal_values(oracle_t *o, const sse_real *u) {
  const sse_config *c = &o->cfg;
  size_t sd = scratch_len(c);
#pragma omp parallel num_threads(o->nthreads)
  {
    sse_real *buf = (sse_real *)malloc(sizeof(sse_real) * sd);
    scratch_t s;
    scratch_carve(c, buf, &s);
#pragma omp for schedule(static)
    for (int k = 0; k < c->n_e; ++k) nodal_values_elem(o, u, k, &s);
    free(buf);
  }
}

void oracle_nodal_values(void *h, const sse_real *u, sse_real *u_q, sse_real *u_f) {
  oracle_t *o = (oracle_t *)h;
  run_nodal_values(o, u);
  if (u_q) memcpy(u_q, o->u_q, sizeof(sse_real) * (size_t)o->cfg.n_q * o->cfg.n_c * o->cfg.n_e);
  if (u_f) memcpy(u_f, o->u_f, sizeof(sse_real) * (size_t)o->cfg.n_f * o->cfg.n_c * o->cfg.n_e);
}

/* semi_discrete_residual! (Threaded), Solvers.jl:495-514 */
void oracle_residual(void *h, const sse_real *u, sse_real *dudt) {
  oracle_t *o = (oracle_t *)h;
  const sse_config *c = &o->cfg;
  run_nodal_values(o, u);
  size_t sd = scratch_len(c);
#pragma omp parallel num_threads(o->nthreads)
  {
    sse_real *buf = (sse_real *)malloc(sizeof(sse_real) * sd);
    scratch_t s;
    scratch_carve(c, buf, &s);
#pragma omp for schedule(static)
    for (int k = 0; k < c->n_e; ++k) {
      if (c->form == SSE_FLUX_DIFFERENCING_FORM) time_derivative_fd(o, dudt, k, &s);
      else time_derivative_standard(o, dudt, k, &s);
    }
    free(buf);
  }
}

/* Carpenter & Kennedy (1994) five-stage fourth-order 2N-storage coefficients */
static const double CK_A[5] = {0.0, -567301805773.0 / 1357537059087.0,
                               -2404267990393.0 / 2016746695238.0,
                               -3550918686646.0 / 2091501179385.0,
                               -1275806237668.0 / 842570457699.0};
static const double CK_B[5] = {1432997174477.0 / 9575080441755.0,
                               5161836677717.0 / 13612068292357.0,
                               1720146321549.0 / 2090206949498.0,
                               3134564353537.0 / 4481467310338.0,
                               2277821191437.0 / 14882151754819.0};

/* fixed-step time integration; scheme 0 = CK2N54 (tmp = A tmp + dt k;
 * u = u + B tmp), scheme 1 = classic RK4 */
void oracle_rk_steps(void *h, sse_real *u, int n_steps, double dt, int scheme) {
  oracle_t *o = (oracle_t *)h;
  const sse_config *c = &o->cfg;
  size_t n = (size_t)c->n_p * c->n_c * c->n_e;
  sse_real *k = (sse_real *)malloc(sizeof(sse_real) * n);
  sse_real *tmp = (sse_real *)malloc(sizeof(sse_real) * n);
  sse_real *acc = scheme == 1 ? (sse_real *)malloc(sizeof(sse_real) * n) : NULL;
  sse_real *ust = scheme == 1 ? (sse_real *)malloc(sizeof(sse_real) * n) : NULL;
  for (int step = 0; step < n_steps; ++step) {
    if (scheme == 0) {
      for (int s = 0; s < 5; ++s) {
        oracle_residual(h, u, k);
        if (s == 0) {
          for (size_t x = 0; x < n; ++x) tmp[x] = dt * k[x];
        } else {
          for (size_t x = 0; x < n; ++x) tmp[x] = CK_A[s] * tmp[x] + dt * k[x];
        }
        for (size_t x = 0; x < n; ++x) u[x] = u[x] + CK_B[s] * tmp[x];
      }
    } else {
      const double half = dt / 2;
      oracle_residual(h, u, k);                                   /* k1 */
      for (size_t x = 0; x < n; ++x) { acc[x] = k[x]; ust[x] = u[x] + half * k[x]; }
      oracle_residual(h, ust, k);                                 /* k2 */
      for (size_t x = 0; x < n; ++x) { acc[x] += 2 * k[x]; ust[x] = u[x] + half * k[x]; }
      oracle_residual(h, ust, k);                                 /* k3 */
      for (size_t x = 0; x < n; ++x) { acc[x] += 2 * k[x]; ust[x] = u[x] + dt * k[x]; }
      oracle_residual(h, ust, k);                                 /* k4 */
      for (size_t x = 0; x < n; ++x) u[x] = u[x] + dt / 6 * (acc[x] + k[x]);
    }
  }
  free(k);
  free(tmp);
  free(acc);
  free(ust);
}

/* Analysis/conservation.jl:145-189.  out[e] = sum_k 1' WJ V dudt[:, e, k];
 * out[N_c] = sum_k w_q' WJ V dudt with w_q the entropy variables of V u
 * (u itself for advection), which equals the reference's
 * (M^-1 V' WJ w_q)' M dudt for both mass solvers. */
void oracle_conservation_residual(void *h, const sse_real *u, const sse_real *dudt, sse_real *out) {
  oracle_t *o = (oracle_t *)h;
  const sse_config *c = &o->cfg;
  const int nq = c->n_q, nc = c->n_c, np = c->n_p;
  for (int e = 0; e <= nc; ++e) out[e] = 0.0;
  sse_real *uq = (sse_real *)malloc(sizeof(sse_real) * nq * nc);
  sse_real *vd = (sse_real *)malloc(sizeof(sse_real) * nq * nc);
  sse_real ui[MAXC], wi[MAXC];
  for (int k = 0; k < c->n_e; ++k) {
    const double *WJ = o->geo.WJ + (size_t)nq * k;
    for (int e = 0; e < nc; ++e) {
      vdm_mul(o, u + (size_t)np * nc * k + np * e, uq + nq * e);
      vdm_mul(o, dudt + (size_t)np * nc * k + np * e, vd + nq * e);
      sse_real s = 0.0;
      for (int i = 0; i < nq; ++i) s += WJ[i] * vd[i + nq * e];
      out[e] += s;
    }
    sse_real s = 0.0;
    for (int i = 0; i < nq; ++i) {
      for (int e = 0; e < nc; ++e) ui[e] = uq[i + nq * e];
      if (c->law == SSE_EULER) cons_to_entropy(c, ui, wi);
      else memcpy(wi, ui, sizeof(sse_real) * nc);
      sse_real t = 0.0;
      for (int e = 0; e < nc; ++e) t += wi[e] * vd[i + nq * e];
      s += WJ[i] * t;
    }
    out[nc] += s;
  }
  free(uq);
  free(vd);
}
