/*
 * Minimal GSL-compatible matrix container for builds where GSL is absent.
 *
 * The reference passes the covariance as a `gsl_matrix *`
 * (src/model_interface.h:23).  The engine reads size1, size2, tda and data.
 * The layout follows the GSL reference manual's description of
 * `gsl_matrix`: size1 (rows), size2 (columns), tda (row stride in
 * elements), data, block, owner.  Elements are row-major:
 * A(i,j) = data[i * tda + j].
 */
#ifndef RG_GSLABI_MATRIX_H
#define RG_GSLABI_MATRIX_H
#include <stddef.h>
#include "gsl_vector.h"
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    size_t size1;
    size_t size2;
    size_t tda;
    double *data;
    gsl_block *block;
    int owner;
} gsl_matrix;

gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2);
gsl_matrix *gsl_matrix_calloc(size_t n1, size_t n2);
void gsl_matrix_free(gsl_matrix *m);
double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j);
void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j, double x);
int gsl_matrix_memcpy(gsl_matrix *dest, const gsl_matrix *src);

#ifdef __cplusplus
}
#endif
#endif
