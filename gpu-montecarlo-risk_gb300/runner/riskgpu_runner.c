/*
 * riskgpu_runner -- C host driver for the drop-in model.
 *
 * Does what the reference's src/main_runner.c does for one "cuda" model
 * (:107-305), without the YAML config, stdin comment and CSV report (those
 * are the reference's reporting plumbing): load the mean vector and
 * covariance written by the reference's preprocessing (format of
 * src/utilities/load_binary.c:5-97: int32 N + N doubles; int32 rows,
 * int32 cols + row-major doubles), fill MonteCarloParams
 * (main_runner.c:168-184), select the model with get_cuda_model()
 * (:230-236), time run_model with CLOCK_MONOTONIC (:244-253), print the
 * results in the format of print_results (:29-35) and free S_values like
 * make_clean (:47-52).
 *
 * usage: riskgpu_runner [-d DATA_DIR] [-M trials] [-k K] [-x X] [-s seed]
 * Defaults are the reference config's (config.yaml:36-41): M=100000000,
 * k=5, x=0.02, seed=67.
 */
#define _POSIX_C_SOURCE 200809L
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#include "riskgpu_plugin.h"

static gsl_vector *load_mu(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "Error: Cannot open %s\n", path); return NULL; }
    int n = 0;
    if (fread(&n, sizeof(int), 1, f) != 1 || n <= 0 || n > 1000000) {
        fprintf(stderr, "Error: bad dimension in %s\n", path);
        fclose(f);
        return NULL;
    }
    gsl_vector *v = gsl_vector_alloc((size_t)n);
    if (!v || fread(v->data, sizeof(double), (size_t)n, f) != (size_t)n) {
        fprintf(stderr, "Error: Failed to read data from %s\n", path);
        gsl_vector_free(v);
        fclose(f);
        return NULL;
    }
    fclose(f);
    return v;
}

static gsl_matrix *load_sigma(const char *path)
{
    FILE *f = fopen(path, "rb");
    if (!f) { fprintf(stderr, "Error: Cannot open %s\n", path); return NULL; }
    int r = 0, c = 0;
    if (fread(&r, sizeof(int), 1, f) != 1 || fread(&c, sizeof(int), 1, f) != 1 || r <= 0 || c <= 0 ||
        (long long)r * c > 2000000000LL) {
        fprintf(stderr, "Error: bad dimensions in %s\n", path);
        fclose(f);
        return NULL;
    }
    gsl_matrix *m = gsl_matrix_alloc((size_t)r, (size_t)c);
    size_t total = (size_t)r * (size_t)c;
    if (!m || fread(m->data, sizeof(double), total, f) != total) {
        fprintf(stderr, "Error: Failed to read data from %s\n", path);
        gsl_matrix_free(m);
        fclose(f);
        return NULL;
    }
    fclose(f);
    return m;
}

int main(int argc, char **argv)
{
    const char *dir = "data";
    long long M = 100000000LL;
    int k = 5;
    double x = 0.02;
    unsigned long seed = 67;
    for (int i = 1; i + 1 < argc; i += 2) {
        if (!strcmp(argv[i], "-d")) dir = argv[i + 1];
        else if (!strcmp(argv[i], "-M")) M = atoll(argv[i + 1]);
        else if (!strcmp(argv[i], "-k")) k = atoi(argv[i + 1]);
        else if (!strcmp(argv[i], "-x")) x = atof(argv[i + 1]);
        else if (!strcmp(argv[i], "-s")) seed = strtoul(argv[i + 1], NULL, 10);
        else { fprintf(stderr, "unknown option %s\n", argv[i]); return 2; }
    }
    char pm[4096], ps[4096];
    snprintf(pm, sizeof pm, "%s/mu.bin", dir);
    snprintf(ps, sizeof ps, "%s/sigma.bin", dir);
    gsl_vector *mu = load_mu(pm);
    gsl_matrix *Sigma = load_sigma(ps);
    if (!mu || !Sigma) {
        gsl_vector_free(mu);
        gsl_matrix_free(Sigma);
        return 1;
    }
    if (M < 1 || M > 2147483647LL) { fprintf(stderr, "Error: M must be in [1, INT_MAX]\n"); return 1; }

    MonteCarloParams params;
    params.N = (int)mu->size;
    params.k = k;
    params.x = x;
    params.M = (int)M;
    params.random_seed = seed;
    params.mu = mu;
    params.Sigma = Sigma;

    MonteCarloResult result;
    memset(&result, 0, sizeof(result));
    ModelFunctions model = get_cuda_model();
    struct timespec t0, t1;
    clock_gettime(CLOCK_MONOTONIC, &t0);
    int status = model.run_model(&params, &result);
    clock_gettime(CLOCK_MONOTONIC, &t1);
    long ms = (long)((t1.tv_sec - t0.tv_sec) * 1000L + (t1.tv_nsec - t0.tv_nsec) / 1000000L);
    int rc = 0;
    if (status == 0) {
        printf("\n%s RESULTS\n", model.name);
        printf("Estimated Probability (P_MIN): %.6f\n", result.P_hat);
        printf("Extreme Events Count: %d out of %d trials\n", result.count, params.M);
        printf("Standard Error: %.6f\n", result.std_error);
        printf("95%% Confidence Interval: [%.6f, %.6f]\n", result.ci_lower, result.ci_upper);
        printf("execution_time_ms: %ld\n", ms);
    } else {
        fprintf(stderr, "Error: %s model failed\n", model.name);
        rc = 1;
    }
    if (result.S_values) {
        free(result.S_values);
        result.S_values = NULL;
    }
    gsl_vector_free(mu);
    gsl_matrix_free(Sigma);
    return rc;
}
