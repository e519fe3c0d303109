// FP64 Cholesky factorisation of the covariance on the GPU.
//
// Replaces the host-side GSL factorisation of the reference wrapper
// (src/05-GPU/monte_carlos_cuda.cu:84-93, gsl_linalg_cholesky_decomp1) and
// its flatten step (:96-108, lower triangle kept, upper zeroed).  FP64 is
// kept for this one step: it is the step whose stability needs it.
//
// One CTA factors the matrix left-looking, column by column, in place in
// the row-major output:
//   L_jj = sqrt(A_jj - sum_{k<j} L_jk^2)
//   L_ij = (A_ij - sum_{k<j} L_ik L_jk) / L_jj,   i > j
// Row j (final once column j-1 is done) is staged in shared memory and read
// by every thread; thread t owns rows i = j+1+t, j+1+t+blockDim, ...
// A pivot that is not > 0 (or not finite) stops the factorisation and
// records info = j + 1; the host turns that into RG_ERR_NOT_PD.  A
// non-finite input records info = -1 (RG_ERR_INVALID).
//
// The same launch then writes the packed FP32 rows used by the fused
// counting kernel and the portfolio moments w^T Sigma w and w.mu (FP64).
#include <cmath>
#include "rg_internal.cuh"

namespace rg {

static constexpr int kCholThreads = 512;
static constexpr int kCholMaxN = 4096; // shared staging of one row: 32 KB

__device__ __forceinline__ double block_sum(double v, double *red)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if (lane == 0) red[warp] = v;
    __syncthreads();
    double t = 0.0;
    if (warp == 0) {
        t = (lane < (int)(blockDim.x >> 5)) ? red[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
        if (lane == 0) red[32] = t;
    }
    __syncthreads();
    return red[32];
}

__global__ void __launch_bounds__(kCholThreads) cholesky_kernel(
    const double *__restrict__ A, long long lda, int n, const double *__restrict__ w,
    const double *__restrict__ mu, double *__restrict__ L, float *__restrict__ Lp,
    float *__restrict__ w32, double *__restrict__ aux, int *__restrict__ info)
{
    extern __shared__ double srow[]; // n doubles
    __shared__ double red[33];
    __shared__ double s_piv;
    __shared__ int s_fail;
    const int tid = threadIdx.x, bs = blockDim.x;

    // Every input that reaches the kernels must be finite (mu, weights, the
    // lower triangle of Sigma); info = -1 reports one that is not.
    int bad = 0;
    for (long long idx = tid; idx < (long long)n * n; idx += bs) {
        const int i = (int)(idx / n), j = (int)(idx % n);
        if (j <= i && !isfinite(A[(long long)i * lda + j])) bad = 1;
    }
    for (int i = tid; i < n; i += bs) {
        if (!isfinite(mu[i])) bad = 1;
        if (w != nullptr && !isfinite(w[i])) bad = 1;
        w32[i] = (w != nullptr) ? (float)w[i] : 0.f;
    }
    if (__syncthreads_or(bad)) {
        if (tid == 0) *info = -1;
        return;
    }

    // Portfolio moments from the input (lower triangle, symmetric use).
    if (w != nullptr) {
        double part = 0.0, pm = 0.0;
        for (long long idx = tid; idx < (long long)n * n; idx += bs) {
            const int i = (int)(idx / n), j = (int)(idx % n);
            const double a = (j <= i) ? A[(long long)i * lda + j] : A[(long long)j * lda + i];
            part += w[i] * a * w[j];
        }
        for (int i = tid; i < n; i += bs) pm += w[i] * mu[i];
        const double wsw = block_sum(part, red);
        const double wmu = block_sum(pm, red);
        if (tid == 0) { aux[0] = wsw; aux[1] = wmu; }
    } else if (tid == 0) {
        aux[0] = 0.0;
        aux[1] = 0.0;
    }

    // L <- lower(A), zero upper.
    for (long long idx = tid; idx < (long long)n * n; idx += bs) {
        const int i = (int)(idx / n), j = (int)(idx % n);
        L[idx] = (j <= i) ? A[(long long)i * lda + j] : 0.0;
    }
    if (tid == 0) s_fail = 0;
    __syncthreads();

    for (int j = 0; j < n; j++) {
        // stage row j (entries k < j are final) and form the pivot
        double part = 0.0;
        for (int k = tid; k < j; k += bs) {
            const double v = L[(long long)j * n + k];
            srow[k] = v;
            part += v * v;
        }
        const double ss = block_sum(part, red); // also orders srow writes before reads
        if (tid == 0) {
            const double d = L[(long long)j * n + j] - ss;
            if (!(d > 0.0) || !isfinite(d)) {
                s_fail = j + 1;
            } else {
                s_piv = sqrt(d);
                L[(long long)j * n + j] = s_piv;
            }
        }
        __syncthreads();
        if (s_fail) break;
        const double piv = s_piv;
        for (int i = j + 1 + tid; i < n; i += bs) {
            const double *row = L + (long long)i * n;
            double s0 = row[j], s1 = 0.0;
            int k = 0;
            for (; k + 1 < j; k += 2) {
                s0 = fma(-row[k], srow[k], s0);
                s1 = fma(-row[k + 1], srow[k + 1], s1);
            }
            if (k < j) s0 = fma(-row[k], srow[k], s0);
            L[(long long)i * n + j] = (s0 + s1) / piv;
        }
        __syncthreads();
    }
    if (tid == 0) *info = s_fail;
    if (s_fail) return;
    __syncthreads();

    // Packed FP32 rows (zero padded to multiples of 4).
    for (int i = tid; i < n; i += bs) {
        const int off = packed_row_offset(i), len = 4 * (i / 4 + 1);
        for (int j = 0; j < len; j++) Lp[off + j] = (j <= i) ? (float)L[(long long)i * n + j] : 0.f;
    }
}

int cholesky_max_n() { return kCholMaxN; }

cudaError_t launch_cholesky(const double *A, long long lda, int n, const double *w,
                            const double *mu, double *L64, float *Lp, float *w32, double *aux,
                            int *info, cudaStream_t s)
{
    if (n > kCholMaxN) return cudaErrorInvalidValue;
    const size_t smem = sizeof(double) * (size_t)(n > 0 ? n : 1);
    if (smem > 48 * 1024) {
        cudaError_t e = cudaFuncSetAttribute(cholesky_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem);
        if (e != cudaSuccess) return e;
    }
    cholesky_kernel<<<1, kCholThreads, smem, s>>>(A, lda, n, w, mu, L64, Lp, w32, aux, info);
    return cudaGetLastError();
}

} // namespace rg
