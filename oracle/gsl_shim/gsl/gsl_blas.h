/*
 * ORACLE TEST INFRASTRUCTURE.  GSL BLAS shim: gsl_blas_dgemv, the one BLAS
 * call the reference makes (monte_carlo_serial.c:72, monte_carlo_omp.c:85).
 * y = alpha*op(A)*x + beta*y with a plain row-by-row loop that sums
 * j = 0..n-1 in order, as the reference CBLAS (gslcblas) does.
 */
#ifndef ORC_GSL_BLAS_H
#define ORC_GSL_BLAS_H
#include <gsl/gsl_matrix.h>
#include <gsl/gsl_vector.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE_t;
int gsl_blas_dgemv(CBLAS_TRANSPOSE_t TransA, double alpha, const gsl_matrix *A,
                   const gsl_vector *X, double beta, gsl_vector *Y);
#ifdef __cplusplus
}
#endif
#endif
