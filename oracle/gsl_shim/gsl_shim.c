/*
 * ORACLE TEST INFRASTRUCTURE -- not part of the engine.  Only the tests,
 * the smoke check and the CPU-baseline leg of the benchmark link this.
 *
 * Self-written stand-in for the parts of GSL 2.7 that the reference's CPU
 * models call (GSL is a third-party dependency of the reference that is not
 * vendored in it and not installed here):
 *   - MT19937 generator: Matsumoto & Nishimura, "Mersenne Twister: a
 *     623-dimensionally equidistributed uniform pseudo-random number
 *     generator", ACM TOMACS 8(1), 1998, with the 2002 initialisation
 *     (init_genrand).  GSL's manual documents gsl_rng_set(r, 0) as using the
 *     generator's default seed, 4357 for mt19937.
 *   - gsl_rng_uniform / _pos: x / 2^32, the _pos form redrawing exact zeros.
 *   - gsl_ran_gaussian: Marsaglia polar method (Knuth TAOCP vol. 2,
 *     3.4.1 Algorithm P); one of the two variates of each accepted pair is
 *     returned, the second is discarded.
 *   - gsl_linalg_cholesky_decomp1: Cholesky-Banachiewicz on the lower
 *     triangle; strict upper triangle left as it was (GSL manual) unless
 *     shim_set_decomp1_keep_upper(0).
 *   - gsl_blas_dgemv: row loop, j ascending, as the reference CBLAS.
 * None of GSL's source is copied; the draw stream is therefore not
 * guaranteed to equal GSL's bit for bit, and comparisons against the
 * reference's published numbers are statistical.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#include <gsl/gsl_rng.h>
#include <gsl/gsl_randist.h>
#include <gsl/gsl_linalg.h>
#include <gsl/gsl_blas.h>

/* ---------------- MT19937 ---------------- */
#define MT_N 624
#define MT_M 397

typedef struct {
    unsigned long mt[MT_N];
    int mti;
} mt_state_t;

static const gsl_rng_type mt_type = {"mt19937", 0xffffffffUL, 0UL, sizeof(mt_state_t)};
const gsl_rng_type *gsl_rng_mt19937 = &mt_type;

static void mt_seed(mt_state_t *s, unsigned long seed)
{
    if (seed == 0) seed = 4357; /* generator default seed */
    s->mt[0] = seed & 0xffffffffUL;
    for (int i = 1; i < MT_N; i++) {
        s->mt[i] = (1812433253UL * (s->mt[i - 1] ^ (s->mt[i - 1] >> 30)) + (unsigned long)i);
        s->mt[i] &= 0xffffffffUL;
    }
    s->mti = MT_N;
}

static unsigned long mt_next(mt_state_t *s)
{
    const unsigned long upper = 0x80000000UL, lower = 0x7fffffffUL, twist = 0x9908b0dfUL;
    unsigned long y;
    if (s->mti >= MT_N) {
        int kk;
        for (kk = 0; kk < MT_N - MT_M; kk++) {
            y = (s->mt[kk] & upper) | (s->mt[kk + 1] & lower);
            s->mt[kk] = s->mt[kk + MT_M] ^ (y >> 1) ^ ((y & 1UL) ? twist : 0UL);
        }
        for (; kk < MT_N - 1; kk++) {
            y = (s->mt[kk] & upper) | (s->mt[kk + 1] & lower);
            s->mt[kk] = s->mt[kk + (MT_M - MT_N)] ^ (y >> 1) ^ ((y & 1UL) ? twist : 0UL);
        }
        y = (s->mt[MT_N - 1] & upper) | (s->mt[0] & lower);
        s->mt[MT_N - 1] = s->mt[MT_M - 1] ^ (y >> 1) ^ ((y & 1UL) ? twist : 0UL);
        s->mti = 0;
    }
    y = s->mt[s->mti++];
    /* tempering */
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680UL;
    y ^= (y << 15) & 0xefc60000UL;
    y ^= (y >> 18);
    return y & 0xffffffffUL;
}

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T)
{
    if (T != gsl_rng_mt19937) return NULL;
    gsl_rng *r = (gsl_rng *)malloc(sizeof(gsl_rng));
    if (!r) return NULL;
    r->type = T;
    r->state = malloc(sizeof(mt_state_t));
    if (!r->state) { free(r); return NULL; }
    mt_seed((mt_state_t *)r->state, 0);
    return r;
}

void gsl_rng_set(const gsl_rng *r, unsigned long seed) { mt_seed((mt_state_t *)r->state, seed); }

void gsl_rng_free(gsl_rng *r)
{
    if (!r) return;
    free(r->state);
    free(r);
}

unsigned long gsl_rng_get(const gsl_rng *r) { return mt_next((mt_state_t *)r->state); }

double gsl_rng_uniform(const gsl_rng *r) { return (double)mt_next((mt_state_t *)r->state) / 4294967296.0; }

double gsl_rng_uniform_pos(const gsl_rng *r)
{
    double u;
    do { u = gsl_rng_uniform(r); } while (u == 0.0);
    return u;
}

/* ---------------- Gaussian: polar method ---------------- */
double gsl_ran_gaussian(const gsl_rng *r, double sigma)
{
    double a, b, q;
    do {
        a = 2.0 * gsl_rng_uniform_pos(r) - 1.0;
        b = 2.0 * gsl_rng_uniform_pos(r) - 1.0;
        q = a * a + b * b;
    } while (q > 1.0 || q == 0.0);
    return sigma * b * sqrt(-2.0 * log(q) / q);
}

/* ---------------- Cholesky (decomp1 semantics) ---------------- */
static int keep_upper_flag = -1; /* -1: not yet read from the environment */

void shim_set_decomp1_keep_upper(int keep) { keep_upper_flag = keep ? 1 : 0; }

int shim_get_decomp1_keep_upper(void)
{
    if (keep_upper_flag < 0) {
        const char *e = getenv("SHIM_DECOMP1_KEEP_UPPER");
        keep_upper_flag = (e && e[0] == '0') ? 0 : 1;
    }
    return keep_upper_flag;
}

int gsl_linalg_cholesky_decomp1(gsl_matrix *A)
{
    const size_t n = A->size1;
    if (A->size2 != n) return 20; /* GSL_ENOTSQR */
    const size_t ld = A->tda;
    double *a = A->data;
    for (size_t i = 0; i < n; i++) {
        for (size_t j = 0; j <= i; j++) {
            double s = a[i * ld + j];
            for (size_t k = 0; k < j; k++) s -= a[i * ld + k] * a[j * ld + k];
            if (i == j) {
                if (!(s > 0.0)) return GSL_EDOM; /* not positive definite (or NaN) */
                a[i * ld + i] = sqrt(s);
            } else {
                a[i * ld + j] = s / a[j * ld + j];
            }
        }
    }
    if (!shim_get_decomp1_keep_upper())
        for (size_t i = 0; i < n; i++)
            for (size_t j = i + 1; j < n; j++) a[i * ld + j] = 0.0;
    return 0;
}

/* ---------------- dgemv ---------------- */
int gsl_blas_dgemv(CBLAS_TRANSPOSE_t TransA, double alpha, const gsl_matrix *A,
                   const gsl_vector *X, double beta, gsl_vector *Y)
{
    const size_t m = A->size1, n = A->size2;
    if (TransA == CblasNoTrans) {
        if (X->size != n || Y->size != m) return 19; /* GSL_EBADLEN */
        for (size_t i = 0; i < m; i++) {
            double t = 0.0;
            for (size_t j = 0; j < n; j++) t += A->data[i * A->tda + j] * X->data[j * X->stride];
            double y = (beta == 0.0) ? 0.0 : beta * Y->data[i * Y->stride];
            Y->data[i * Y->stride] = y + alpha * t;
        }
    } else {
        if (X->size != m || Y->size != n) return 19;
        for (size_t j = 0; j < n; j++) {
            double t = 0.0;
            for (size_t i = 0; i < m; i++) t += A->data[i * A->tda + j] * X->data[i * X->stride];
            double y = (beta == 0.0) ? 0.0 : beta * Y->data[j * Y->stride];
            Y->data[j * Y->stride] = y + alpha * t;
        }
    }
    return 0;
}
