/*
 * ORACLE TEST INFRASTRUCTURE.  GSL linear-algebra shim: the one call the
 * reference makes, gsl_linalg_cholesky_decomp1 (monte_carlo_serial.c:37,
 * monte_carlo_omp.c:48, monte_carlos_cuda.cu:88).
 *
 * Semantics follow the GSL 2.7 manual for decomp1: the lower triangle and
 * diagonal of A are read, L overwrites them, and the strict upper triangle
 * is left unmodified.  Because the reference's CPU models then pass the
 * whole matrix to gsl_blas_dgemv, the untouched upper triangle changes
 * their returns; shim_set_decomp1_keep_upper(0) zeroes it instead so the
 * mathematically intended R = mu + L Z can be checked too.  The
 * environment variable SHIM_DECOMP1_KEEP_UPPER=0|1 sets the same switch.
 * A non-positive pivot returns GSL_EDOM (1) without aborting.
 */
#ifndef ORC_GSL_LINALG_H
#define ORC_GSL_LINALG_H
#include <gsl/gsl_matrix.h>
#ifdef __cplusplus
extern "C" {
#endif
#define GSL_EDOM 1
int gsl_linalg_cholesky_decomp1(gsl_matrix *A);
void shim_set_decomp1_keep_upper(int keep);
int shim_get_decomp1_keep_upper(void);
#ifdef __cplusplus
}
#endif
#endif
