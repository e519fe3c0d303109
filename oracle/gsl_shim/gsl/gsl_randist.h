/*
 * ORACLE TEST INFRASTRUCTURE.  GSL random-distribution shim: the one call
 * the reference makes, gsl_ran_gaussian (monte_carlo_serial.c:68,
 * monte_carlo_omp.c:79).  Implemented with the Marsaglia polar form of the
 * Box-Muller method (Knuth, TAOCP vol. 2, 3.4.1 Algorithm P), the method
 * GSL 2.7 documents for this call.
 */
#ifndef ORC_GSL_RANDIST_H
#define ORC_GSL_RANDIST_H
#include "gsl_rng.h"
#ifdef __cplusplus
extern "C" {
#endif
double gsl_ran_gaussian(const gsl_rng *r, double sigma);
#ifdef __cplusplus
}
#endif
#endif
