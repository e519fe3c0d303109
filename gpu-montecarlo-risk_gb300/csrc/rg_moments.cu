// Preprocessing on the GPU: the sample moments of a daily-returns matrix and
// the realised crash frequency, in FP64.
//
// Replaces the reference's offline pandas steps:
//   compute_stats   preprocessing/preprocessing_stats.py:18,21
//                   mu = train.mean(), Sigma = train.cov() (ddof = 1)
//   compute_metrics preprocessing/evaluation.py:19,22
//                   fraction of days with (returns < -x).sum() >= k
//
// Moments, two passes like pandas' own covariance (means first, then the
// sum of products of deviations):
//   col_mean   one thread per column, rows in order, Kahan-compensated;
//   cov_tile   one CTA per 32 x 32 tile of the lower triangle of Sigma
//              (diagonal tiles in full), rows in chunks of 32 staged
//              centred in shared memory; each tile is written at (i, j) and
//              mirrored to (j, i).
// Every output is summed in a fixed order, so results do not depend on
// scheduling.  The work is T N^2 / 2 FP64 FMAs (about 3.6e8 for 600 assets
// and 2000 days), spread over all SMs.
#include <cmath>
#include <cstring>
#include "rg_internal.cuh"

namespace rg {

static constexpr int kMomTile = 32;

__global__ void col_mean_kernel(const double *__restrict__ X, long long T, int n, long long ld,
                                double *__restrict__ mu)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= n) return;
    double s = 0.0, c = 0.0;
    for (long long t = 0; t < T; t++) {
        const double y = X[t * ld + j] - c;
        const double u = s + y;
        c = (u - s) - y;
        s = u;
    }
    mu[j] = s / (double)T;
}

__global__ void __launch_bounds__(256) cov_tile_kernel(const double *__restrict__ X, long long T, int n, long long ld,
                                                       const double *__restrict__ mu, double *__restrict__ S)
{
    __shared__ double A[kMomTile][kMomTile + 1], B[kMomTile][kMomTile + 1];
    const int t = blockIdx.x;
    int bi = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f);
    while ((bi + 1) * (bi + 2) / 2 <= t) bi++;
    while (bi * (bi + 1) / 2 > t) bi--;
    const int bj = t - bi * (bi + 1) / 2;
    const int i0 = bi * kMomTile, j0 = bj * kMomTile;
    const int r = threadIdx.x >> 3, cb = (threadIdx.x & 7) * 4;
    double acc[4] = {0.0, 0.0, 0.0, 0.0};
    for (long long t0 = 0; t0 < T; t0 += kMomTile) {
        for (int e = threadIdx.x; e < kMomTile * kMomTile; e += blockDim.x) {
            const int tt = e / kMomTile, cc = e % kMomTile;
            const bool row_ok = t0 + tt < T;
            A[tt][cc] = (row_ok && i0 + cc < n) ? X[(t0 + tt) * ld + i0 + cc] - mu[i0 + cc] : 0.0;
            B[tt][cc] = (row_ok && j0 + cc < n) ? X[(t0 + tt) * ld + j0 + cc] - mu[j0 + cc] : 0.0;
        }
        __syncthreads();
#pragma unroll 8
        for (int tt = 0; tt < kMomTile; tt++) {
            const double a = A[tt][r];
#pragma unroll
            for (int u = 0; u < 4; u++) acc[u] = fma(a, B[tt][cb + u], acc[u]);
        }
        __syncthreads();
    }
    const int gi = i0 + r;
    if (gi >= n) return;
    const double inv = 1.0 / (double)(T - 1);
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int gj = j0 + cb + u;
        if (gj >= n) continue;
        const double v = acc[u] * inv;
        S[(long long)gi * n + gj] = v;
        if (bi != bj) S[(long long)gj * n + gi] = v;
    }
}

__global__ void crash_days_kernel(const double *__restrict__ X, long long T, int n, long long ld, double neg_x,
                                  int k, unsigned long long *__restrict__ days)
{
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (t >= T) return;
    const double *row = X + t * ld;
    int c = 0;
    for (int j = 0; j < n; j++) c += (row[j] < neg_x) ? 1 : 0;
    if (c >= k) atomicAdd(days, 1ull);
}

} // namespace rg

using namespace rg;

namespace {

int check_matrix(const double *X, int64_t T, int32_t n, int64_t ld, int64_t min_rows)
{
    if (!X) return set_error(RG_ERR_INVALID, "returns is NULL");
    if (n < 1) return set_error(RG_ERR_INVALID, "n must be >= 1 (got %d)", n);
    if (T < min_rows) return set_error(RG_ERR_INVALID, "need at least %lld rows (got %lld)", (long long)min_rows, (long long)T);
    if (ld < n) return set_error(RG_ERR_INVALID, "ld (%lld) must be >= n (%d)", (long long)ld, n);
    for (int64_t t = 0; t < T; t++)
        for (int32_t j = 0; j < n; j++)
            if (!std::isfinite(X[t * ld + j]))
                return set_error(RG_ERR_INVALID, "returns[%lld][%d] is not finite", (long long)t, j);
    return RG_OK;
}

int device_ready()
{
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count <= 0) {
        cudaGetLastError();
        return set_error(RG_ERR_NO_DEVICE, "no CUDA device is available");
    }
    return RG_OK;
}

} // namespace

extern "C" int rg_moments(const double *returns, int64_t T, int32_t n, int64_t ld, double *mu_out, double *sigma_out,
                          void *stream)
{
    int st = check_matrix(returns, T, n, ld, 2);
    if (st != RG_OK) return st;
    if (!mu_out || !sigma_out) return set_error(RG_ERR_INVALID, "mu_out / sigma_out is NULL");
    if ((st = device_ready()) != RG_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    double *dX = nullptr, *dmu = nullptr, *dS = nullptr;
    const size_t xbytes = (size_t)T * (size_t)n * sizeof(double);
    const int nb = (n + kMomTile - 1) / kMomTile;
    cudaError_t e = cudaMalloc(&dX, xbytes);
    if (e == cudaSuccess) e = cudaMalloc(&dmu, (size_t)n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dS, (size_t)n * n * sizeof(double));
    // rows packed to width n on the device
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(dX, (size_t)n * sizeof(double), returns, (size_t)ld * sizeof(double),
                              (size_t)n * sizeof(double), (size_t)T, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) {
        col_mean_kernel<<<(n + 127) / 128, 128, 0, s>>>(dX, T, n, n, dmu);
        cov_tile_kernel<<<nb * (nb + 1) / 2, 256, 0, s>>>(dX, T, n, n, dmu, dS);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(mu_out, dmu, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(sigma_out, dS, (size_t)n * n * sizeof(double), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dX);
    cudaFree(dmu);
    cudaFree(dS);
    if (e != cudaSuccess)
        return set_error(e == cudaErrorMemoryAllocation ? RG_ERR_NOMEM : RG_ERR_CUDA, "rg_moments: %s",
                         cudaGetErrorString(e));
    return RG_OK;
}

extern "C" int rg_crash_frequency(const double *returns, int64_t T, int32_t n, int64_t ld, double x, int32_t k,
                                  double *freq_out, void *stream)
{
    int st = check_matrix(returns, T, n, ld, 1);
    if (st != RG_OK) return st;
    if (!freq_out) return set_error(RG_ERR_INVALID, "freq_out is NULL");
    if (!std::isfinite(x)) return set_error(RG_ERR_INVALID, "x must be finite");
    if ((st = device_ready()) != RG_OK) return st;
    cudaStream_t s = (cudaStream_t)stream;
    double *dX = nullptr;
    unsigned long long *dcount = nullptr, days = 0;
    cudaError_t e = cudaMalloc(&dX, (size_t)T * (size_t)n * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc(&dcount, sizeof(unsigned long long));
    if (e == cudaSuccess)
        e = cudaMemcpy2DAsync(dX, (size_t)n * sizeof(double), returns, (size_t)ld * sizeof(double),
                              (size_t)n * sizeof(double), (size_t)T, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), s);
    if (e == cudaSuccess) {
        crash_days_kernel<<<(unsigned)((T + 255) / 256), 256, 0, s>>>(dX, T, n, n, -x, k, dcount);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(&days, dcount, sizeof(days), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    cudaFree(dX);
    cudaFree(dcount);
    if (e != cudaSuccess)
        return set_error(e == cudaErrorMemoryAllocation ? RG_ERR_NOMEM : RG_ERR_CUDA, "rg_crash_frequency: %s",
                         cudaGetErrorString(e));
    *freq_out = (double)days / (double)T;
    return RG_OK;
}
