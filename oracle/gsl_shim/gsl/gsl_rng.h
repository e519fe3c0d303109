/*
 * ORACLE TEST INFRASTRUCTURE.  GSL random-number-generator shim.
 *
 * GSL 2.7 (the version the reference's cluster scripts load,
 * gpu_script.sh:27) is not installed here.  This header declares the few
 * generator calls the reference's CPU models make
 * (src/02-C-serial/monte_carlo_serial.c:46,54,68,91;
 * src/03-openMP/monte_carlo_omp.c:57,66,79):
 *   gsl_rng_alloc(gsl_rng_mt19937), gsl_rng_set, gsl_rng_free,
 *   gsl_rng_uniform_pos, gsl_rng_get.
 * The generator is MT19937 as published by Matsumoto & Nishimura (1998),
 * seeded the way GSL's manual describes gsl_rng_set for mt19937 (seed 0 is
 * replaced by the default seed 4357).
 */
#ifndef ORC_GSL_RNG_H
#define ORC_GSL_RNG_H
#define RG_GSLABI_RNG_H /* suppress the engine's type-only stand-in */
#ifdef __cplusplus
extern "C" {
#endif

typedef struct gsl_rng_type {
    const char *name;
    unsigned long max;
    unsigned long min;
    unsigned long size;
} gsl_rng_type;

typedef struct {
    const gsl_rng_type *type;
    void *state;
} gsl_rng;

extern const gsl_rng_type *gsl_rng_mt19937;

gsl_rng *gsl_rng_alloc(const gsl_rng_type *T);
void gsl_rng_set(const gsl_rng *r, unsigned long seed);
void gsl_rng_free(gsl_rng *r);
unsigned long gsl_rng_get(const gsl_rng *r);
double gsl_rng_uniform(const gsl_rng *r);
double gsl_rng_uniform_pos(const gsl_rng *r);

#ifdef __cplusplus
}
#endif
#endif
