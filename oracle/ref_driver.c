/*
 * ORACLE TEST INFRASTRUCTURE.  Thin driver that runs the reference's own CPU
 * models -- src/02-C-serial/monte_carlo_serial.c and
 * src/03-openMP/monte_carlo_omp.c, compiled unmodified from the reference
 * tree against the GSL shim -- through the reference plugin API
 * (src/model_interface.h:9-36), the same way src/main_runner.c:168-184,248
 * fills MonteCarloParams and calls run_model.  Built only where the
 * reference sources exist (oracle/Makefile, target _ref/libref_cpu.so); the
 * result pins the oracle's restatement to the reference's own code.
 */
#include <stdlib.h>
#include <string.h>
#include <omp.h>
#include <gsl/gsl_vector.h>
#include <gsl/gsl_matrix.h>
#include <gsl/gsl_linalg.h>
#include "model_interface.h"

extern ModelFunctions get_serial_model(void);
extern ModelFunctions get_openmp_model(void);

/* Thread count of the OpenMP model (its omp_get_max_threads, monte_carlo_omp.c:36). */
void ref_set_threads(int n)
{
    if (n > 0) omp_set_num_threads(n);
}

/* model: 0 = serial, 1 = openmp.  S_out (nullable) receives M values.
 * out6 = {P_hat, count, std_error, ci_lower, ci_upper, status}. */
int ref_run(int model, int n, const double *mu, const double *sigma, int M, int k, double x,
            unsigned long seed, int keep_upper, int *S_out, double out6[6])
{
    shim_set_decomp1_keep_upper(keep_upper);
    MonteCarloParams params;
    MonteCarloResult result;
    memset(&result, 0, sizeof(result));
    params.x = x;
    params.N = n;
    params.k = k;
    params.M = M;
    params.random_seed = seed;
    params.mu = gsl_vector_alloc((size_t)n);
    params.Sigma = gsl_matrix_alloc((size_t)n, (size_t)n);
    memcpy(params.mu->data, mu, sizeof(double) * (size_t)n);
    memcpy(params.Sigma->data, sigma, sizeof(double) * (size_t)n * (size_t)n);
    ModelFunctions f = model == 0 ? get_serial_model() : get_openmp_model();
    int status = f.run_model(&params, &result);
    if (status == 0 && S_out && result.S_values) memcpy(S_out, result.S_values, sizeof(int) * (size_t)M);
    out6[0] = result.P_hat;
    out6[1] = (double)result.count;
    out6[2] = result.std_error;
    out6[3] = result.ci_lower;
    out6[4] = result.ci_upper;
    out6[5] = (double)status;
    free(result.S_values);
    gsl_vector_free(params.mu);
    gsl_matrix_free(params.Sigma);
    return status;
}
