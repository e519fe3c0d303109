/*
 * riskgpu -- GB300 (sm_103a) Monte Carlo portfolio-risk engine, C ABI.
 *
 * Plain C types and pointers only.  Every entry point returns an rg_status
 * (0 = success, negative = error class); rg_last_error() gives the message
 * of the calling thread's last failure.  Streams are passed as `void *`
 * holding a cudaStream_t (NULL = the engine's own stream).
 *
 * Model (the reference's, src/01-python-serial/python_serial.py:3-7 and
 * src/05-GPU/monte_carlos_cuda.cu:23-72, extended by portfolio weights and
 * a horizon): for each path p,
 *     Zsum = sum_{d<H} Z_d,  Z_d ~ N(0, I_N)
 *     R    = H mu + L Zsum,  L L^T = Sigma (FP64 Cholesky on the GPU)
 *     S    = #{ i : R_i < -x }            crash count   (reference)
 *     crash  if S >= k                     (reference's extreme event)
 *     breach if w.R < port_threshold       (portfolio extension)
 * plus VaR / CVaR of the loss -w.R.  Counts are exact 64-bit integers.
 */
#ifndef RISKGPU_H
#define RISKGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define RG_ABI_VERSION 1

typedef enum {
    RG_OK = 0,
    RG_ERR_INVALID = -1,     /* bad argument (sizes, NaN/Inf inputs, null pointers) */
    RG_ERR_NOT_PD = -2,      /* covariance not positive definite (Cholesky pivot <= 0) */
    RG_ERR_CUDA = -3,        /* a CUDA runtime call or kernel failed */
    RG_ERR_NOMEM = -4,       /* device or host allocation failed */
    RG_ERR_UNSUPPORTED = -5, /* valid request this build cannot serve (size limits) */
    RG_ERR_ADMISSION = -6,   /* refused: not enough free device memory headroom */
    RG_ERR_NO_DEVICE = -7,   /* no usable CUDA device */
    RG_ERR_TIMEOUT = -8,     /* a bounded device wait ran out (error word set on device) */
    RG_ERR_BUSY = -9         /* queue full / handle in use */
} rg_status;

/* Normal-draw layout. */
typedef enum {
    /* Counter-based Philox4x32-10, key = seed, counter = (block, 0, path):
     * the same 32-bit stream as cuRAND's curand_init(seed, path, 0) for
     * curandStatePhilox4_32_10_t.  Normals by Box-Muller in FP32. */
    RG_RNG_PHILOX = 0,
    /* The reference kernel's own stream (monte_carlos_cuda.cu:30-31,45-47):
     * curand_init(seed, path, 0, &curandStateXORWOW_t) then
     * curand_normal_double per asset, rounded to FP32. */
    RG_RNG_XORWOW_REF = 1
} rg_rng_layout;

/* How the H daily draws of an asset are formed. */
typedef enum {
    /* H daily N(0,1) draws summed per asset (the model as stated). */
    RG_DRAWS_DAILY = 0,
    /* One N(0,1) draw per asset scaled by sqrt(H): the same N(0, H)
     * distribution of the sum, H times fewer normals, different draws. */
    RG_DRAWS_AGGREGATED = 1
} rg_draw_mode;

/* Arithmetic of the correlation step R = H mu + L Zsum. */
typedef enum {
    RG_PREC_FP32 = 0,   /* FP32 FMA cores (the plain fused kernels) */
    RG_PREC_BF16X3 = 1, /* tcgen05 tensor cores: BF16 hi+lo split of Z and L, three products,
                           FP32 accumulation (about 2^-16 relative per product) */
    RG_PREC_AUTO = 2,   /* the engine picks (currently the FP32 kernels) */
    RG_PREC_FP16X3 = 3  /* tcgen05 tensor cores: FP16 hi+lo split (L scaled by 2^8), three
                           products, FP32 accumulation (close to FP32 rounding) */
} rg_precision;

/* Flags for rg_portfolio_create. */
#define RG_INPUT_DEVICE 0x1 /* mu, sigma, weights are device pointers */

typedef struct rg_portfolio rg_portfolio; /* opaque: device-resident factor */

typedef struct {
    int32_t n_assets;
    int32_t has_weights;
    const double *d_L;      /* device, row-major n x n FP64, zero upper triangle */
    const void *d_packed;   /* device, FP32 packed lower rows (engine layout) */
    double wsw;             /* w^T Sigma w (daily variance of the portfolio return) */
    double wmu;             /* w . mu */
    float ms_cholesky;      /* device time of the Cholesky at creation */
} rg_portfolio_info;

typedef struct {
    int64_t n_paths;        /* M >= 1 */
    uint64_t path_offset;   /* first path index (restartable / shardable ranges) */
    uint64_t seed;
    int32_t horizon;        /* H >= 1 days, draws summed */
    int32_t k;              /* crash count threshold (S >= k) */
    double x;               /* asset crash threshold, R_i < -x */
    double port_threshold;  /* portfolio breach, w.R < port_threshold */
    int32_t rng;            /* rg_rng_layout */
    int32_t precision;      /* rg_precision */
    double var_level;       /* e.g. 0.99; 0 disables VaR/CVaR */
    int32_t *d_s_values;    /* optional device output [n_paths]: S per path */
    float *d_port_values;   /* optional device output [n_paths]: w.R per path */
    int32_t draw_mode;      /* rg_draw_mode */
    int32_t reserved;       /* 0 */
} rg_query;

typedef struct {
    int64_t n_paths;
    int64_t crash_count;    /* #{S >= k} */
    int64_t breach_count;   /* #{w.R < port_threshold} */
    double p_crash, se_crash, ci_lower, ci_upper; /* estimator statistics (reference A8) */
    double p_breach, se_breach;
    double var, cvar;       /* loss quantile / tail mean at var_level */
    int64_t tail_count;     /* number of paths in the VaR tail */
    int32_t var_passes;     /* 1 = single pass, 2 = band missed and a second pass ran */
    float ms_device;        /* device time of the simulation kernels */
} rg_result;

/* ---------------- library ---------------- */
int rg_abi_version(void);
const char *rg_status_string(int status);
const char *rg_last_error(void);
/* Number of CUDA devices visible (0 when none); never fails. */
int rg_device_count(void);

/* ---------------- resident portfolios ---------------- */
/* Uploads mu [n], sigma [n x n, leading dimension ld], weights [n] (nullable)
 * and factors sigma in FP64 on the GPU.  Replaces the host Cholesky and the
 * flatten/copy of the reference wrapper (monte_carlos_cuda.cu:84-122). */
int rg_portfolio_create(int32_t n, const double *mu, const double *sigma, int64_t ld,
                        const double *weights, int32_t flags, rg_portfolio **out);
int rg_portfolio_destroy(rg_portfolio *p);
int rg_portfolio_info_get(const rg_portfolio *p, rg_portfolio_info *out);
/* Copies the FP64 factor L (row-major, zero upper) to host memory. */
int rg_portfolio_factor(const rg_portfolio *p, double *L_host);

/* ---------------- simulation ---------------- */
/* Runs one query to completion and fills `out` (replaces the kernel launch,
 * copy-back and statistics of monte_carlos_cuda.cu:124-150). */
int rg_simulate(const rg_portfolio *p, const rg_query *q, rg_result *out, void *stream);
/* Enqueues only the fused counting kernel on `stream`: d_counts (device,
 * 2 x uint64: crash, breach) are zeroed and accumulated; no host sync, no
 * VaR.  For callers that keep inputs and outputs resident. */
int rg_launch_counts(const rg_portfolio *p, const rg_query *q, unsigned long long *d_counts,
                     void *stream);

/* One-shot from host buffers: create, simulate, destroy. */
int rg_run(int32_t n, const double *mu, const double *sigma, int64_t ld, const double *weights,
           const rg_query *q, rg_result *out);

/* Estimator statistics shared by every back-end of the reference
 * (monte_carlos_cuda.cu:146-150): p = count/M, se = sqrt(p(1-p)/M),
 * 95% CI p -+ 1.96 se clamped to [0,1]. */
void rg_estimator_stats(int64_t count, int64_t M, double *p, double *se, double *lo, double *hi);

/* VaR tail size used by the engine: ceil((1-level) M), clamped to [1, M]. */
int64_t rg_tail_count(int64_t M, double level);

/* ---------------- batches: many queries, one persistent launch ---------------- */
/* No counterpart in the reference (one model run per call,
 * src/main_runner.c:198-298).  A batch holds up to thousands of
 * (portfolio, query) items of uneven N, H and path counts; one launch of
 * the persistent tensor-core kernel computes all of them, CTAs claiming
 * work units of 64-path tiles from a device counter.  The launch (counter
 * resets, kernel, copy of the counts to pinned host memory) is captured
 * once into a CUDA graph and replayed by rg_batch_launch.  Items use the
 * Philox layout, N <= 640, precision FP16X3 (BF16X3 if asked), no VaR. */
typedef struct rg_batch rg_batch;
typedef struct {
    const rg_portfolio *portfolio;
    rg_query query;
} rg_batch_item;
typedef struct {
    int32_t items;
    int64_t total_tiles;   /* 64-path tiles over all items */
    int32_t unit_tiles;    /* tiles per work unit */
    int32_t ctas_per_sm;
    int32_t grid;
    int32_t graph;         /* 1 = replayed from a captured CUDA graph */
    int32_t tuned;         /* 1 = parameters from the autotuner */
    float last_ms;         /* device time of the last launch */
} rg_batch_info;
#define RG_BATCH_NO_GRAPH 0x1 /* launch without graph capture */
int rg_batch_create(const rg_batch_item *items, int32_t count, int32_t flags, rg_batch **out);
int rg_batch_launch(rg_batch *b, void *stream);
/* Waits for the last launch and fills results[count] (no VaR fields). */
int rg_batch_wait(rg_batch *b, rg_result *results);
int rg_batch_info_get(const rg_batch *b, rg_batch_info *out);
/* Autotuner: times every (tiles per unit, CTAs per SM) candidate for this
 * batch's shape class, keeps the fastest for this batch and records it in
 * the JSON cache (RG_TUNE_CACHE, default ./riskgpu_tune.json) that later
 * batches of the class read at creation. */
int rg_batch_tune(rg_batch *b, void *stream);
int rg_batch_destroy(rg_batch *b);

/* ---------------- served form: request loop with continuous batching ---------------- */
/* No counterpart in the reference.  A server keeps registered portfolios
 * resident and runs a scheduler thread: requests that arrive are admitted
 * while free HBM (cudaMemGetInfo) stays above headroom_bytes, packed into
 * one of `slots` preallocated, graph-captured persistent batches (up to
 * max_batch_items requests each) and launched while earlier batches may
 * still be running; completions are polled every poll_us.  A request's
 * result does not depend on the batch that carried it (draws are keyed by
 * seed and path index).  Requests use the Philox layout, N <= 639, no VaR;
 * the portfolios stay owned by the caller and must outlive the server. */
typedef struct rg_server rg_server;
typedef struct {
    int32_t slots;               /* batches in flight on the GPU (default 3) */
    int32_t max_batch_items;     /* requests per batch (default 64) */
    int64_t headroom_bytes;      /* admission: free HBM must exceed this (default 1 GiB) */
    double admission_timeout_ms; /* pending longer than this without headroom: RG_ERR_ADMISSION */
    int32_t poll_us;             /* completion polling interval while work is in flight */
} rg_server_config;
typedef struct {
    int64_t completed;
    int64_t refused;
    int64_t batches;
    double mean_batch_items;
    double p50_ms, p99_ms, max_ms; /* submit-to-result latency of completed requests */
    double paths_per_s;            /* paths completed / (last completion - first submit) */
} rg_server_summary;
void rg_server_default_config(rg_server_config *cfg);
int rg_server_create(const rg_server_config *cfg, rg_server **out);
int rg_server_register(rg_server *s, int32_t portfolio_id, const rg_portfolio *p);
int rg_server_submit(rg_server *s, int32_t portfolio_id, const rg_query *q, uint64_t *ticket);
/* Blocks until the request is done; latency_ms (nullable) = submit to result. */
int rg_server_wait(rg_server *s, uint64_t ticket, rg_result *out, double *latency_ms);
int rg_server_stats(rg_server *s, rg_server_summary *out);
int rg_server_reset_stats(rg_server *s);
int rg_server_destroy(rg_server *s);

/* ---------------- simulation without allocation ---------------- */
/* No counterpart in the reference.  rg_simulate() with no allocation at all,
 * for callers that cannot call cudaMalloc where they run a query: a host
 * that accounts for every device byte itself, a latency-critical loop where
 * an allocation could synchronise the device, a plugin inside a framework
 * whose allocator owns the device heap.  The portfolio (created beforehand)
 * and the query are the inputs, `out` the output; the per-query scratch
 * (counters, VaR histogram, VaR candidates) lives in a 1 MiB device array
 * that every GPU loading this library holds until the process exits.
 *  - Queries whose VaR band could need more than the array's ~253k
 *    candidate slots (about n_paths > 2.5e8 at level 0.99) are rejected with
 *    RG_ERR_UNSUPPORTED and a message naming the limit.
 *  - The first call on each device looks up the array's device address
 *    (cudaGetSymbolAddress, with that device current); make that first call
 *    before any stream capture.
 *  - Calls share the one array: calls whose GPU work overlaps (different
 *    streams or host threads) race on it and must be serialised.
 *  - `stream` NULL means the default stream; ms_device is left 0. */
int rg_simulate_noalloc(const rg_portfolio *p, const rg_query *q, rg_result *out, void *stream);

/* ---------------- preprocessing (daily returns -> mu, Sigma) ---------------- */
/* Sample moments of a daily-returns matrix on the GPU, in FP64:
 * mu_j = mean of column j; Sigma = sum_t (X_t - mu)(X_t - mu)^T / (T - 1)
 * (ddof = 1), full symmetric, row-major n x n.  Replaces compute_stats
 * (preprocessing/preprocessing_stats.py:18,21: pandas train.mean() and
 * train.cov()).  `returns` is a T x n row-major HOST array with leading
 * dimension ld >= n, T >= 2, every entry finite; mu_out (n) and sigma_out
 * (n * n) are host arrays.  Synchronous on `stream` (NULL: default). */
int rg_moments(const double *returns, int64_t T, int32_t n, int64_t ld, double *mu_out, double *sigma_out,
               void *stream);

/* Fraction of the T rows (days) on which at least k of the n returns are
 * below -x.  Replaces compute_metrics (preprocessing/evaluation.py:19,22).
 * Same array conventions as rg_moments (T >= 1). */
int rg_crash_frequency(const double *returns, int64_t T, int32_t n, int64_t ld, double x, int32_t k,
                       double *freq_out, void *stream);

/* ---------------- measurement ---------------- */
/* Roofline denominators of the fused kernels, measured on the current
 * device with micro-kernels timed by CUDA events on `stream`: FP32 FMA
 * throughput and the engine's normal-generation throughput.  (No
 * counterpart in the reference, which has no measurement code.) */
typedef struct {
    double fp32_tflops;
    double normals_per_s;
    int32_t sm_count;
} rg_peaks;
int rg_probe_peaks(rg_peaks *out, void *stream);

#ifdef __cplusplus
}
#endif
#endif /* RISKGPU_H */
