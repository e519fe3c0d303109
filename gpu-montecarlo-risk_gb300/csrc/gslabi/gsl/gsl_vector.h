/*
 * Minimal GSL-compatible vector container for builds where GSL is absent.
 *
 * The reference plugin API (src/model_interface.h:4-6) passes the mean
 * vector as a `gsl_vector *`.  The engine only reads three fields of it
 * (size, stride, data), so the layout below follows the structure that the
 * GSL reference manual documents for `gsl_vector` (size, stride, data,
 * block, owner) and for `gsl_block` (size, data).  A caller compiled
 * against the real GSL hands the engine the same layout.
 *
 * Only the container calls that the reference host code makes are
 * declared: alloc/free/get/set (src/main_runner.c:40,
 * src/utilities/load_binary.c:29, src/05-GPU/monte_carlos_cuda.cu:97).
 */
#ifndef RG_GSLABI_VECTOR_H
#define RG_GSLABI_VECTOR_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    size_t size;
    double *data;
} gsl_block;

typedef struct {
    size_t size;
    size_t stride;
    double *data;
    gsl_block *block;
    int owner;
} gsl_vector;

gsl_vector *gsl_vector_alloc(size_t n);
gsl_vector *gsl_vector_calloc(size_t n);
void gsl_vector_free(gsl_vector *v);
double gsl_vector_get(const gsl_vector *v, size_t i);
void gsl_vector_set(gsl_vector *v, size_t i, double x);
int gsl_vector_add(gsl_vector *a, const gsl_vector *b);

#ifdef __cplusplus
}
#endif
#endif
