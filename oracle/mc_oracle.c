/*
 * ORACLE TEST INFRASTRUCTURE -- NOT THE ENGINE.
 *
 * CPU restatement, in FP64, of the reference's Monte Carlo crash estimator
 * and of the engine's own counter-based sampling layout.  Only the tests,
 * the smoke check and the CPU-baseline leg of the benchmark may load this
 * library; the engine never calls it and has no CPU fallback.
 *
 * What is restated, and from where (paths inside the reference project):
 *   orc_serial_estimate  src/02-C-serial/monte_carlo_serial.c:98-164
 *                        (Cholesky :36-37, MT19937 :46,54, N gaussians
 *                        :67-69, full dgemv :72, +mu :73, count :76-81,
 *                        S>=k :140-142, statistics :152-158)
 *   orc_omp_estimate     src/03-openMP/monte_carlo_omp.c:111-200
 *                        (one shared generator inside `omp critical`
 *                        :77-82, static schedule + reduction :152)
 *   orc_kernel_from_normals
 *                        src/05-GPU/monte_carlos_cuda.cu:23-72 and :96-108:
 *                        lower-triangular L with a zeroed upper triangle,
 *                        R_i = mu_i + sum_{j<=i} L_ij Z_j accumulated from
 *                        0.0 in j order with fused multiply-adds (what nvcc
 *                        emits for `sum += d_L[i*N+j] * Z[j]`), S = #{R_i<-x}.
 *                        The normals come from the caller (on the GPU they
 *                        are cuRAND's, see oracle/xorwow_normals.cu).
 *   orc_stats            the shared estimator statistics (.cu:146-150 =
 *                        monte_carlo_serial.c:152-158): P = count/M,
 *                        SE = sqrt(P(1-P)/M), 95% CI clamped to [0,1].
 *   orc_philox4x32_10 / orc_mc_philox
 *                        the engine's sampling layout restated in FP64:
 *                        Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
 *                        random numbers: as easy as 1, 2, 3", SC'11) with key
 *                        = 64-bit seed and counter = (block, 0, path lo, path
 *                        hi), block = day*ceil(N/4) + asset/4; Box-Muller
 *                        (Box & Muller 1958) on each pair of words; H daily
 *                        draws summed per asset; R = H*mu + L*sum(Z).
 *   orc_factor_crash_prob
 *                        FP64 P(S >= k) for a factor covariance
 *                        Sigma = B B^T + diag(idio^2) and an H-day horizon
 *                        with summed daily draws: R = H mu + sqrt(H)(B F +
 *                        idio e) in distribution, F ~ N(0, I_nf), e ~ N(0, I_n).
 *                        Given F the crashes are independent with
 *                        p_i(F) = Phi((-x - H mu_i - sqrt(H) B_i.F)/(sqrt(H) idio_i)),
 *                        and P(S >= k | F) is the upper tail of a
 *                        Poisson-binomial law (recursion over the assets on
 *                        the counts 0..k-1 with ">= k" absorbing).  The
 *                        caller supplies the factor points F (randomised
 *                        quasi-Monte Carlo) and averages over randomisations.
 *                        No counterpart in the reference (its estimator is
 *                        plain Monte Carlo); it is the FP64 answer that the
 *                        sampled estimates are compared with.
 * Compile with -ffp-contract=off so results do not depend on whether the
 * host compiler fuses multiply-adds (explicit fma() is used where the GPU
 * form being mirrored fuses).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#include <gsl/gsl_rng.h>
#include <gsl/gsl_randist.h>
#include <gsl/gsl_linalg.h>
#include <gsl/gsl_blas.h>
#include <gsl/gsl_matrix.h>
#include <gsl/gsl_vector.h>

typedef struct {
    long long count;
    double P_hat;
    double std_error;
    double ci_lower;
    double ci_upper;
} orc_result;

void orc_stats(long long count, long long M, orc_result *r)
{
    r->count = count;
    r->P_hat = (double)count / (double)M;
    r->std_error = sqrt(r->P_hat * (1.0 - r->P_hat) / (double)M);
    double margin = 1.96 * r->std_error;
    r->ci_lower = fmax(0.0, r->P_hat - margin);
    r->ci_upper = fmin(1.0, r->P_hat + margin);
}

/* Plain FP64 Cholesky of the lower triangle of row-major A (leading
 * dimension lda); L is written row-major n x n with a zero upper triangle.
 * Returns 0, or j+1 for the first non-positive pivot j. */
int orc_cholesky_lower(int n, const double *A, long long lda, double *L)
{
    for (int i = 0; i < n; i++)
        for (int j = 0; j < n; j++) L[(size_t)i * n + j] = 0.0;
    for (int i = 0; i < n; i++) {
        for (int j = 0; j <= i; j++) {
            double s = A[(size_t)i * lda + j];
            for (int k = 0; k < j; k++) s -= L[(size_t)i * n + k] * L[(size_t)j * n + k];
            if (i == j) {
                if (!(s > 0.0)) return j + 1;
                L[(size_t)i * n + i] = sqrt(s);
            } else {
                L[(size_t)i * n + j] = s / L[(size_t)j * n + j];
            }
        }
    }
    return 0;
}

static gsl_matrix *sigma_to_gsl(int n, const double *sigma)
{
    gsl_matrix *m = gsl_matrix_alloc((size_t)n, (size_t)n);
    if (!m) return NULL;
    memcpy(m->data, sigma, sizeof(double) * (size_t)n * (size_t)n);
    return m;
}

/* Restatement of serial_simulate.  keep_upper selects what the Cholesky
 * leaves above the diagonal before the full-matrix dgemv (1 = GSL decomp1
 * semantics, the reference's actual arithmetic; 0 = pure L). */
int orc_serial_estimate(int n, const double *mu, const double *sigma, long long M, int k, double x,
                        unsigned long seed, int keep_upper, int *S_out, orc_result *res)
{
    shim_set_decomp1_keep_upper(keep_upper);
    gsl_matrix *L = sigma_to_gsl(n, sigma);
    if (!L) return -1;
    if (gsl_linalg_cholesky_decomp1(L)) { gsl_matrix_free(L); return -1; }
    gsl_rng *rng = gsl_rng_alloc(gsl_rng_mt19937);
    gsl_rng_set(rng, seed);
    gsl_vector *Z = gsl_vector_alloc((size_t)n), *R = gsl_vector_alloc((size_t)n);
    gsl_vector *vmu = gsl_vector_alloc((size_t)n);
    for (int i = 0; i < n; i++) gsl_vector_set(vmu, (size_t)i, mu[i]);
    long long count = 0;
    for (long long p = 0; p < M; p++) {
        for (int i = 0; i < n; i++) gsl_vector_set(Z, (size_t)i, gsl_ran_gaussian(rng, 1.0));
        gsl_blas_dgemv(CblasNoTrans, 1.0, L, Z, 0.0, R);
        gsl_vector_add(R, vmu);
        int S = 0;
        for (int i = 0; i < n; i++) S += (gsl_vector_get(R, (size_t)i) < -x);
        if (S_out) S_out[p] = S;
        if (S >= k) count++;
    }
    gsl_vector_free(Z); gsl_vector_free(R); gsl_vector_free(vmu);
    gsl_rng_free(rng); gsl_matrix_free(L);
    orc_stats(count, M, res);
    return 0;
}

/* Restatement of openmp_simulate: one generator shared by every thread and
 * drawn from inside a critical section, trials split statically.  Each
 * critical section takes the N draws of one trial, so the set of normal
 * vectors equals the serial run's and the total count matches it, while
 * which trial receives which vector depends on the interleaving. */
int orc_omp_estimate(int n, const double *mu, const double *sigma, long long M, int k, double x,
                     unsigned long seed, int keep_upper, int nthreads, orc_result *res)
{
    shim_set_decomp1_keep_upper(keep_upper);
    gsl_matrix *L = sigma_to_gsl(n, sigma);
    if (!L) return -1;
    if (gsl_linalg_cholesky_decomp1(L)) { gsl_matrix_free(L); return -1; }
    gsl_rng *rng = gsl_rng_alloc(gsl_rng_mt19937);
    gsl_rng_set(rng, seed);
    gsl_vector *vmu = gsl_vector_alloc((size_t)n);
    for (int i = 0; i < n; i++) gsl_vector_set(vmu, (size_t)i, mu[i]);
    long long count = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel
    {
        gsl_vector *Z = gsl_vector_alloc((size_t)n), *R = gsl_vector_alloc((size_t)n);
#pragma omp for reduction(+ : count) schedule(static)
        for (long long p = 0; p < M; p++) {
#pragma omp critical
            {
                for (int i = 0; i < n; i++) gsl_vector_set(Z, (size_t)i, gsl_ran_gaussian(rng, 1.0));
            }
            gsl_blas_dgemv(CblasNoTrans, 1.0, L, Z, 0.0, R);
            gsl_vector_add(R, vmu);
            int S = 0;
            for (int i = 0; i < n; i++) S += (gsl_vector_get(R, (size_t)i) < -x);
            if (S >= k) count++;
        }
        gsl_vector_free(Z); gsl_vector_free(R);
    }
    gsl_vector_free(vmu); gsl_rng_free(rng); gsl_matrix_free(L);
    orc_stats(count, M, res);
    return 0;
}

/* The reference GPU kernel's arithmetic in FP64, given its normals.
 * L is row-major n x n, lower triangle used.  Z is M x n (path-major).
 * R_out (nullable) receives the M x n returns. */
long long orc_kernel_from_normals(int n, const double *mu, const double *L, long long M,
                                  const double *Z, double x, int k, int *S_out, double *R_out)
{
    long long count = 0;
    for (long long p = 0; p < M; p++) {
        const double *z = Z + (size_t)p * n;
        int S = 0;
        for (int i = 0; i < n; i++) {
            double sum = 0.0;
            for (int j = 0; j <= i; j++) sum = fma(L[(size_t)i * n + j], z[j], sum);
            double r = mu[i] + sum;
            if (R_out) R_out[(size_t)p * n + i] = r;
            S += (r < -x);
        }
        if (S_out) S_out[p] = S;
        if (S >= k) count++;
    }
    return count;
}

/* ---------------- Philox4x32-10 ---------------- */
void orc_philox4x32_10(const uint32_t ctr_in[4], const uint32_t key_in[2], uint32_t out[4])
{
    uint32_t c0 = ctr_in[0], c1 = ctr_in[1], c2 = ctr_in[2], c3 = ctr_in[3];
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int r = 0; r < 10; r++) {
        uint64_t p0 = (uint64_t)0xD2511F53u * c0;
        uint64_t p1 = (uint64_t)0xCD9E8D57u * c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c0 = hi1 ^ c1 ^ k0;
        c1 = lo1;
        c2 = hi0 ^ c3 ^ k1;
        c3 = lo0;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* The engine's 23-bit fraction of a word: f = 1 + (w >> 9) 2^-23 in [1, 2)
 * (exact in FP32 and FP64). */
static inline double engine_one_to_two(uint32_t w) { return 1.0 + (double)(w >> 9) * 0x1p-23; }

/* Box-Muller on one pair of 32-bit words, in FP64 from the engine's
 * uniforms u_a = 2 - f(a) in (0, 1] and angle t = 2 pi f(b) in [2 pi, 4 pi):
 * z0 = r cos(t), z1 = r sin(t), r = sqrt(-2 ln u_a). */
static inline void box_muller(uint32_t a, uint32_t b, double *z0, double *z1)
{
    const double two_pi = 6.283185307179586476925286766559;
    double ua = 2.0 - engine_one_to_two(a);
    double r = sqrt(-2.0 * log(ua));
    double t = two_pi * engine_one_to_two(b);
    *z0 = r * cos(t);
    *z1 = r * sin(t);
}

/* Normals of one path in the engine's layout: out[d*n + j] for day d,
 * asset j (n_days x n values). */
void orc_philox_normals(uint64_t seed, uint64_t path, int n, int n_days, double *out)
{
    const int nq = (n + 3) / 4;
    uint32_t key[2] = {(uint32_t)seed, (uint32_t)(seed >> 32)};
    for (int d = 0; d < n_days; d++) {
        for (int q = 0; q < nq; q++) {
            uint32_t ctr[4] = {(uint32_t)(d * nq + q), 0u, (uint32_t)path, (uint32_t)(path >> 32)};
            uint32_t w[4];
            double z[4];
            orc_philox4x32_10(ctr, key, w);
            box_muller(w[0], w[1], &z[0], &z[1]);
            box_muller(w[2], w[3], &z[2], &z[3]);
            for (int e = 0; e < 4; e++) {
                int j = 4 * q + e;
                if (j < n) out[(size_t)d * n + j] = z[e];
            }
        }
    }
}

/* FP64 Monte Carlo in the engine's layout.  L row-major n x n (lower
 * triangle read), w may be NULL (no portfolio), paths are
 * path_offset .. path_offset+M-1.  Per-path outputs are nullable.
 * counts[0] = #{S >= k}, counts[1] = #{w.R < port_threshold}.
 * aggregated = 1: one draw per asset scaled by sqrt(H) instead of the sum of
 * H daily draws (the engine's RG_DRAWS_AGGREGATED). */
void orc_mc_philox(int n, const double *mu, const double *L, const double *w, int n_days,
                   long long M, uint64_t path_offset, uint64_t seed, double x, int k,
                   double port_threshold, int *S_out, double *port_out, double *R_out,
                   long long counts[2], int nthreads, int aggregated)
{
    long long crash = 0, breach = 0;
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#else
    (void)nthreads;
#endif
#pragma omp parallel reduction(+ : crash, breach)
    {
        double *z = (double *)malloc(sizeof(double) * (size_t)n * (size_t)n_days);
        double *zs = (double *)malloc(sizeof(double) * (size_t)n);
#pragma omp for schedule(static)
        for (long long p = 0; p < M; p++) {
            if (aggregated) {
                /* one N(0,1) draw per asset (day 0 of the layout) times sqrt(H) */
                orc_philox_normals(seed, path_offset + (uint64_t)p, n, 1, z);
                for (int j = 0; j < n; j++) zs[j] = sqrt((double)n_days) * z[j];
            } else {
                orc_philox_normals(seed, path_offset + (uint64_t)p, n, n_days, z);
                for (int j = 0; j < n; j++) {
                    double s = 0.0;
                    for (int d = 0; d < n_days; d++) s += z[(size_t)d * n + j];
                    zs[j] = s;
                }
            }
            int S = 0;
            double port = 0.0;
            for (int i = 0; i < n; i++) {
                double r = (double)n_days * mu[i];
                for (int j = 0; j <= i; j++) r += L[(size_t)i * n + j] * zs[j];
                if (R_out) R_out[(size_t)p * n + i] = r;
                S += (r < -x);
                if (w) port += w[i] * r;
            }
            if (S_out) S_out[p] = S;
            if (port_out) port_out[p] = port;
            if (S >= k) crash++;
            if (w && port < port_threshold) breach++;
        }
        free(z);
        free(zs);
    }
    counts[0] = crash;
    counts[1] = breach;
}


/* Mean over the npts factor points F (npts x nf, row-major) of
 * P(S >= k | F), see the header.  Points are split in fixed contiguous
 * ranges per thread and the partial sums added in thread order, so the
 * result does not depend on scheduling. */
double orc_factor_crash_prob(int n, int nf, int horizon, const double *mu, const double *B,
                             const double *idio, double x, int k, long long npts, const double *F,
                             int nthreads)
{
    if (n < 1 || nf < 1 || k < 1 || npts < 1) return NAN;
    if (k > n) return 0.0;
    const double H = (double)horizon, sh = sqrt(H);
    int nt = 1;
#ifdef _OPENMP
    nt = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
    (void)nthreads;
#endif
    double *part = (double *)calloc((size_t)nt, sizeof(double));
    if (!part) return NAN;
#pragma omp parallel num_threads(nt)
    {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        const long long lo = npts * t / nt, hi = npts * (t + 1) / nt;
        double *d = (double *)malloc(sizeof(double) * (size_t)(k + 1));
        double acc = 0.0;
        for (long long q = lo; q < hi && d; q++) {
            const double *f = F + q * nf;
            for (int j = 0; j <= k; j++) d[j] = 0.0;
            d[0] = 1.0;
            for (int i = 0; i < n; i++) {
                double bf = 0.0;
                for (int c = 0; c < nf; c++) bf += B[(size_t)i * nf + c] * f[c];
                const double z = (-x - H * mu[i] - sh * bf) / (sh * idio[i]);
                const double p = 0.5 * erfc(-z / sqrt(2.0));
                const double r = 1.0 - p;
                d[k] += d[k - 1] * p;
                for (int j = k - 1; j >= 1; j--) d[j] = d[j] * r + d[j - 1] * p;
                d[0] *= r;
            }
            acc += d[k];
        }
        free(d);
        part[t] = acc;
    }
    double sum = 0.0;
    for (int t = 0; t < nt; t++) sum += part[t];
    free(part);
    return sum / (double)npts;
}
