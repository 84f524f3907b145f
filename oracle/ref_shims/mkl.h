/*
 * Stand-in for the one MKL routine the reference's omega path calls
 * (cblas_dgemm, source_beta_to_omega/src/calc.c:639,651,667-679), used ONLY to
 * compile the reference into the test oracle (oracle/_ref).  Test
 * infrastructure.  Sequential, like the reference's -lmkl_sequential link
 * (source_beta_to_omega/makefile:15-17).
 */
#ifndef SCLET_ORACLE_MKL_SHIM_H
#define SCLET_ORACLE_MKL_SHIM_H

typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;

void cblas_dgemm(CBLAS_LAYOUT layout, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb,
                 int m, int n, int k, double alpha, const double *a, int lda,
                 const double *b, int ldb, double beta, double *c, int ldc);

#endif
