/*
 * Type-only stand-in for GSL's random number generator header.
 *
 * The reference plugin header includes <gsl/gsl_rng.h> (src/model_interface.h:4)
 * but the plugin structures never use a generator.  This declares the
 * generator type with the two-field layout the GSL manual describes
 * (type, state) so that the header compiles where GSL is absent.  The
 * oracle ships a full generator in its own header of the same name.
 */
#ifndef RG_GSLABI_RNG_H
#define RG_GSLABI_RNG_H
#ifdef __cplusplus
extern "C" {
#endif
typedef struct gsl_rng_type gsl_rng_type;
typedef struct {
    const gsl_rng_type *type;
    void *state;
} gsl_rng;
#ifdef __cplusplus
}
#endif
#endif
