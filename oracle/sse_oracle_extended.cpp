/*
 * sse_oracle_extended.cpp -- TEST INFRASTRUCTURE ONLY: the CPU restatement
 * in sse_oracle.c evaluated in extended precision (long double: 64-bit
 * mantissa on x86-64, IEEE binary128 on AArch64), the reference against
 * which the FP64 residuals (the CUDA library's and the FP64 oracle's own)
 * are measured.  Where the residual is a small difference of large flux
 * contributions, an FP64 evaluation carries a relative error well above
 * 1e-16 whatever its summation order; comparing both FP64 evaluations with
 * this one separates that inherent cancellation from any error of the
 * library's own.  Nothing in the product links or calls it.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/sse_gb300.h"

#define SSE_ORACLE_REAL long double
namespace extended {
#include "sse_oracle.c"
}

namespace {
size_t state_len(void *h) {
  const sse_config &c = ((extended::oracle_t *)h)->cfg;
  return (size_t)c.n_p * c.n_c * c.n_e;
}
}  // namespace

extern "C" {

void *oracle_extended_create(const sse_config *cfg, const sse_operators *ops, const sse_geometry *geo,
                             int nthreads) {
  return extended::oracle_create(cfg, ops, geo, nthreads);
}

void oracle_extended_destroy(void *h) { extended::oracle_destroy(h); }

/* dudt = R(u), evaluated in long double, rounded to double at the end */
void oracle_extended_residual(void *h, const double *u, double *dudt) {
  const size_t n = state_len(h);
  long double *x = (long double *)malloc(sizeof(long double) * (n ? n : 1));
  long double *y = (long double *)malloc(sizeof(long double) * (n ? n : 1));
  for (size_t i = 0; i < n; ++i) x[i] = u[i];
  extended::oracle_residual(h, x, y);
  for (size_t i = 0; i < n; ++i) dudt[i] = (double)y[i];
  free(x);
  free(y);
}

/* the number of mantissa bits of the extended type */
int oracle_extended_digits(void) { return (int)__LDBL_MANT_DIG__; }

}  // extern "C"
