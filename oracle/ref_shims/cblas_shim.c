/*
 * Column-major, no-transpose DGEMM: C = alpha*A*B + beta*C.  The only form the
 * reference calls (source_beta_to_omega/src/calc.c:639,651,667-679).  Test
 * infrastructure for oracle/_ref.  Each output column is accumulated over k in
 * ascending order (the textbook definition of the product).
 */
#include "mkl.h"

#include <stdio.h>
#include <stdlib.h>

void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb,
                 int m, int n, int k, double alpha, const double *a, int lda,
                 const double *b, int ldb, double beta, double *c, int ldc) {
  int i, j, l;
  if (layout != CblasColMajor || ta != CblasNoTrans || tb != CblasNoTrans) {
    fprintf(stderr, "cblas shim: only ColMajor/NoTrans/NoTrans is supported\n");
    exit(3);
  }
  for (j = 0; j < n; j++) {
    double *cj = c + (size_t)j * ldc;
    const double *bj = b + (size_t)j * ldb;
    if (beta == 0.0) {
      for (i = 0; i < m; i++) cj[i] = 0.0;
    } else if (beta != 1.0) {
      for (i = 0; i < m; i++) cj[i] *= beta;
    }
    for (l = 0; l < k; l++) {
      const double s = alpha * bj[l];
      const double *al = a + (size_t)l * lda;
      for (i = 0; i < m; i++) cj[i] += al[i] * s;
    }
  }
}
