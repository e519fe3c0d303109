/*
 * riskgpu drop-in for the reference's C plugin API.
 *
 * The structures below are layout-identical to the reference's
 * src/model_interface.h:9-36 so that a host compiled against either header
 * can call this engine.  The include guard is the reference header's own
 * (MODEL_INTERFACE_H): whichever of the two a translation unit includes
 * first defines the types, the other is skipped.
 *
 * GSL types: the structures hold `gsl_vector *` / `gsl_matrix *`.  With GSL
 * installed these come from GSL; without it the engine ships a minimal
 * layout-compatible container layer (csrc/gslabi).  The engine itself only
 * reads size/stride/data and size1/size2/tda/data.
 */
#ifndef RISKGPU_PLUGIN_H
#define RISKGPU_PLUGIN_H

#ifndef MODEL_INTERFACE_H
#define MODEL_INTERFACE_H
#include <gsl/gsl_rng.h>
#include <gsl/gsl_vector.h>
#include <gsl/gsl_matrix.h>

/* src/model_interface.h:9-16 */
typedef struct {
    double P_hat;     /* count / M */
    int count;        /* #{S >= k}, saturated at INT_MAX */
    int *S_values;    /* malloc'ed by the model, freed by the caller; NULL unless
                         RG_MATERIALIZE_S=1 (see cuda_simulate) */
    double std_error;
    double ci_lower;
    double ci_upper;
} MonteCarloResult;

/* src/model_interface.h:19-27 */
typedef struct {
    double x;
    int N;
    int k;
    gsl_vector *mu;
    gsl_matrix *Sigma;
    int M;
    unsigned long random_seed;
} MonteCarloParams;

/* src/model_interface.h:30 */
typedef int (*ModelRunFunc)(MonteCarloParams *params, MonteCarloResult *result);

/* src/model_interface.h:33-36 */
typedef struct {
    const char *name;
    ModelRunFunc run_model;
} ModelFunctions;
#endif /* MODEL_INTERFACE_H */

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces src/05-GPU/monte_carlos_cuda.cu:165-171: returns
 * { .name = "cuda", .run_model = cuda_simulate }.  src/main_runner.c:24-26,
 * 230-236 binds it when built with -DCUDA_BUILD. */
ModelFunctions get_cuda_model(void);

/* Replaces src/05-GPU/monte_carlos_cuda.cu:75-163.  Same contract: reads
 * params (owned by the caller), fills result, returns 0 or -1 with a message
 * on stderr.  N is not limited to 64.  Behaviour switches (environment):
 *   RG_RNG=xorwow      draw the reference kernel's own cuRAND XORWOW stream
 *                      (default: Philox, the engine's counter-based layout)
 *   RG_MATERIALIZE_S=1 fill result->S_values (host malloc, M ints) as the
 *                      reference does; by default no per-path data leaves
 *                      the GPU and S_values stays NULL. */
int cuda_simulate(MonteCarloParams *params, MonteCarloResult *result);

#ifdef __cplusplus
}
#endif
#endif /* RISKGPU_PLUGIN_H */
