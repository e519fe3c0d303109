/*
 * Container functions for the minimal GSL-compatible layer (gsl/gsl_vector.h,
 * gsl/gsl_matrix.h).  Written from the behaviour the GSL reference manual
 * documents: alloc returns uninitialised storage, calloc zeroed storage,
 * free releases block and struct, get/set index with the stride or tda.
 * Only linked into host drivers built where GSL is absent; the engine
 * library itself never calls these.
 */
#include <stdlib.h>
#include <string.h>
#include "gsl/gsl_vector.h"
#include "gsl/gsl_matrix.h"

static gsl_block *block_new(size_t n, int zero)
{
    gsl_block *b = (gsl_block *)malloc(sizeof(gsl_block));
    if (!b) return NULL;
    b->size = n;
    b->data = (double *)(zero ? calloc(n ? n : 1, sizeof(double))
                              : malloc((n ? n : 1) * sizeof(double)));
    if (!b->data) { free(b); return NULL; }
    return b;
}

static gsl_vector *vector_new(size_t n, int zero)
{
    gsl_vector *v = (gsl_vector *)malloc(sizeof(gsl_vector));
    if (!v) return NULL;
    v->block = block_new(n, zero);
    if (!v->block) { free(v); return NULL; }
    v->size = n;
    v->stride = 1;
    v->data = v->block->data;
    v->owner = 1;
    return v;
}

gsl_vector *gsl_vector_alloc(size_t n) { return vector_new(n, 0); }
gsl_vector *gsl_vector_calloc(size_t n) { return vector_new(n, 1); }

void gsl_vector_free(gsl_vector *v)
{
    if (!v) return;
    if (v->owner && v->block) { free(v->block->data); free(v->block); }
    free(v);
}

double gsl_vector_get(const gsl_vector *v, size_t i) { return v->data[i * v->stride]; }
void gsl_vector_set(gsl_vector *v, size_t i, double x) { v->data[i * v->stride] = x; }

int gsl_vector_add(gsl_vector *a, const gsl_vector *b)
{
    if (a->size != b->size) return 19; /* GSL_EBADLEN */
    for (size_t i = 0; i < a->size; i++) a->data[i * a->stride] += b->data[i * b->stride];
    return 0;
}

static gsl_matrix *matrix_new(size_t n1, size_t n2, int zero)
{
    gsl_matrix *m = (gsl_matrix *)malloc(sizeof(gsl_matrix));
    if (!m) return NULL;
    m->block = block_new(n1 * n2, zero);
    if (!m->block) { free(m); return NULL; }
    m->size1 = n1;
    m->size2 = n2;
    m->tda = n2;
    m->data = m->block->data;
    m->owner = 1;
    return m;
}

gsl_matrix *gsl_matrix_alloc(size_t n1, size_t n2) { return matrix_new(n1, n2, 0); }
gsl_matrix *gsl_matrix_calloc(size_t n1, size_t n2) { return matrix_new(n1, n2, 1); }

void gsl_matrix_free(gsl_matrix *m)
{
    if (!m) return;
    if (m->owner && m->block) { free(m->block->data); free(m->block); }
    free(m);
}

double gsl_matrix_get(const gsl_matrix *m, size_t i, size_t j) { return m->data[i * m->tda + j]; }
void gsl_matrix_set(gsl_matrix *m, size_t i, size_t j, double x) { m->data[i * m->tda + j] = x; }

int gsl_matrix_memcpy(gsl_matrix *dest, const gsl_matrix *src)
{
    if (dest->size1 != src->size1 || dest->size2 != src->size2) return 19; /* GSL_EBADLEN */
    for (size_t i = 0; i < src->size1; i++)
        memcpy(dest->data + i * dest->tda, src->data + i * src->tda, src->size2 * sizeof(double));
    return 0;
}
