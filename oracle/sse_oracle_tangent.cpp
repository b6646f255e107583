/*
 * sse_oracle_tangent.cpp -- TEST INFRASTRUCTURE ONLY: forward-mode
 * (dual-number) derivatives of the CPU restatement in sse_oracle.c, the
 * checker for the CUDA library's discrete adjoint.  Nothing in the product
 * links or calls it.
 *
 * sse_oracle.c is compiled a second time, as C++, with its scalar type
 * sse_real set to a dual number (value, tangent).  Every arithmetic
 * operation and math function carries the exact derivative along, so the
 * tangent part of oracle_residual(u + eps v) is J(u) v and that of
 * oracle_rk_steps is the directional derivative of the whole trajectory --
 * the role ForwardDiff plays through the reference's CPU residual.  The
 * adjoint is checked against it by the dot-product identity
 * <lam, J v> = <J^T lam, v>, which holds to round-off.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/sse_gb300.h"

struct sse_dual {
  double v, d;
  sse_dual() : v(0.0), d(0.0) {}
  sse_dual(double x) : v(x), d(0.0) {}  // NOLINT: constants promote implicitly
  sse_dual(double x, double dx) : v(x), d(dx) {}
  sse_dual &operator+=(const sse_dual &b) { v += b.v; d += b.d; return *this; }
  sse_dual &operator-=(const sse_dual &b) { v -= b.v; d -= b.d; return *this; }
  sse_dual &operator*=(const sse_dual &b) { d = d * b.v + v * b.d; v *= b.v; return *this; }
};

static inline sse_dual operator+(const sse_dual &a, const sse_dual &b) { return {a.v + b.v, a.d + b.d}; }
static inline sse_dual operator-(const sse_dual &a, const sse_dual &b) { return {a.v - b.v, a.d - b.d}; }
static inline sse_dual operator-(const sse_dual &a) { return {-a.v, -a.d}; }
static inline sse_dual operator*(const sse_dual &a, const sse_dual &b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }
static inline sse_dual operator/(const sse_dual &a, const sse_dual &b) {
  const double q = a.v / b.v;
  return {q, (a.d - q * b.d) / b.v};
}
static inline bool operator<(const sse_dual &a, const sse_dual &b) { return a.v < b.v; }
static inline bool operator>(const sse_dual &a, const sse_dual &b) { return a.v > b.v; }
static inline bool operator<=(const sse_dual &a, const sse_dual &b) { return a.v <= b.v; }
static inline bool operator>=(const sse_dual &a, const sse_dual &b) { return a.v >= b.v; }

// math functions with their derivatives
static inline sse_dual log(const sse_dual &a) { return {::log(a.v), a.d / a.v}; }
static inline sse_dual exp(const sse_dual &a) {
  const double e = ::exp(a.v);
  return {e, e * a.d};
}
static inline sse_dual sqrt(const sse_dual &a) {
  const double r = ::sqrt(a.v);
  return {r, a.d / (2.0 * r)};
}
static inline sse_dual pow(const sse_dual &a, double g) {
  return {::pow(a.v, g), g * ::pow(a.v, g - 1.0) * a.d};
}
static inline sse_dual fabs(const sse_dual &a) { return a.v < 0.0 ? -a : a; }
static inline sse_dual fmax(const sse_dual &a, const sse_dual &b) { return a.v >= b.v ? a : b; }
// fma: the value keeps the fused rounding of the double build
static inline sse_dual fma(const sse_dual &a, const sse_dual &b, const sse_dual &c) {
  return {::fma(a.v, b.v, c.v), a.d * b.v + a.v * b.d + c.d};
}

#define SSE_ORACLE_REAL sse_dual
namespace tangent {
#include "sse_oracle.c"
}

namespace {
sse_dual *to_dual(const double *x, const double *dx, size_t n) {
  sse_dual *y = (sse_dual *)malloc(sizeof(sse_dual) * (n ? n : 1));
  for (size_t i = 0; i < n; ++i) y[i] = sse_dual(x[i], dx ? dx[i] : 0.0);
  return y;
}
void from_dual(const sse_dual *y, double *x, double *dx, size_t n) {
  for (size_t i = 0; i < n; ++i) {
    if (x) x[i] = y[i].v;
    if (dx) dx[i] = y[i].d;
  }
}
size_t state_len(void *h) {
  const sse_config &c = ((tangent::oracle_t *)h)->cfg;
  return (size_t)c.n_p * c.n_c * c.n_e;
}
}  // namespace

extern "C" {

void *oracle_tangent_create(const sse_config *cfg, const sse_operators *ops, const sse_geometry *geo,
                            int nthreads) {
  return tangent::oracle_create(cfg, ops, geo, nthreads);
}

void oracle_tangent_destroy(void *h) { tangent::oracle_destroy(h); }

/* dudt = R(u), jv = J(u) v */
void oracle_tangent_residual(void *h, const double *u, const double *v, double *dudt, double *jv) {
  const size_t n = state_len(h);
  sse_dual *x = to_dual(u, v, n), *y = to_dual(u, nullptr, n);
  tangent::oracle_residual(h, x, y);
  from_dual(y, dudt, jv, n);
  free(x);
  free(y);
}

/* u <- u(T), v <- (du(T)/du(0)) v over n_steps fixed steps */
void oracle_tangent_rk_steps(void *h, double *u, double *v, int n_steps, double dt, int scheme) {
  const size_t n = state_len(h);
  sse_dual *x = to_dual(u, v, n);
  tangent::oracle_rk_steps(h, x, n_steps, dt, scheme);
  from_dual(x, u, v, n);
  free(x);
}

}  // extern "C"
