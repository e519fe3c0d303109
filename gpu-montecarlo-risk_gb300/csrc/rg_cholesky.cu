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
//
// Above kCholSingleMaxN a blocked right-looking form spreads the work over
// the SMs (one SM's FP64 rate is a small fraction of the part's): for each
// 32-column block k,
//   chol_diag    one warp factors the diagonal block in registers,
//   chol_panel   one thread per row solves L_ik L_kk^T = A_ik below it,
//   chol_update  one CTA per 32 x 32 tile of the trailing lower triangle
//                subtracts L_ik L_jk^T,
// between chol_prep (finite checks, lower(A), w32, per-row moment terms)
// and chol_finish (packed FP32 rows, moment sums in a fixed order, so the
// result does not depend on scheduling).  The first pivot that is not > 0
// (or not finite) records info = column + 1 and every later kernel returns
// at once.
#include <cmath>
#include <cstdlib>
#include <cstring>
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

// ------------------------------------------------------------ blocked form
static constexpr int kCholNb = 32;          // block size (one warp per diagonal block)
static constexpr int kCholSingleMaxN = 64;  // the single-CTA form up to here

// Checks, L <- lower(A) (upper zeroed), w32, and the per-row moment terms
// aux[2 + i] = w_i sum_j Sigma_ij w_j, aux[2 + n + i] = w_i mu_i.  One warp
// per row.
__global__ void chol_prep_kernel(const double *__restrict__ A, long long lda, int n, const double *__restrict__ w,
                                 const double *__restrict__ mu, double *__restrict__ L, float *__restrict__ w32,
                                 double *__restrict__ aux, int *__restrict__ info)
{
    const int lane = threadIdx.x & 31;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    int bad = 0;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const double *ai = A + (long long)i * lda;
        double part = 0.0;
        for (int j = lane; j < n; j += 32) {
            const double a = (j <= i) ? ai[j] : A[(long long)j * lda + i];
            if (j <= i && !isfinite(a)) bad = 1;
            L[(long long)i * n + j] = (j <= i) ? a : 0.0;
            if (w != nullptr) part += a * w[j];
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
        if (lane == 0) {
            if (!isfinite(mu[i]) || (w != nullptr && !isfinite(w[i]))) bad = 1;
            w32[i] = (w != nullptr) ? (float)w[i] : 0.f;
            aux[2 + i] = (w != nullptr) ? w[i] * part : 0.0;
            aux[2 + n + i] = (w != nullptr) ? w[i] * mu[i] : 0.0;
        }
    }
    if (bad) atomicExch(info, -1);
}

// Factor the diagonal block at k0 (kb <= 32 columns) with one warp; lane r
// holds row r of the block in registers (fully unrolled), and column values
// move between lanes by shuffles.  Right-looking: after column c is scaled,
// lane r subtracts L_rc L_jc from its entries j in (c, r].
__global__ void chol_diag_kernel(double *__restrict__ L, int n, int k0, int kb, int *__restrict__ info)
{
    if (*info != 0) return;
    const int r = threadIdx.x;
    double a[kCholNb];
#pragma unroll
    for (int c = 0; c < kCholNb; c++) a[c] = (r < kb && c <= r) ? L[(long long)(k0 + r) * n + k0 + c] : 0.0;
#pragma unroll
    for (int c = 0; c < kCholNb; c++) {
        if (c < kb) {
            const double d = __shfl_sync(0xffffffffu, a[c], c); // the same value in every lane: uniform branch
            if (!(d > 0.0) || !isfinite(d)) {
                if (r == 0) *info = k0 + c + 1;
                return;
            }
            // one FP64 reciprocal square root per column instead of a square
            // root and a division: both are long FP64 sequences on this part
            const double rs = rsqrt(d);
            if (r == c) a[c] = d * rs;
            if (r > c) a[c] = a[c] * rs;
#pragma unroll
            for (int j = c + 1; j < kCholNb; j++) {
                const double ljc = __shfl_sync(0xffffffffu, a[c], j);
                if (r >= j) a[j] = fma(-a[c], ljc, a[j]);
            }
        }
    }
    if (r < kb) {
#pragma unroll
        for (int c = 0; c < kCholNb; c++)
            if (c <= r) L[(long long)(k0 + r) * n + k0 + c] = a[c];
    }
}

// Rows below the diagonal block: x L_kk^T = a, one thread per row (32 per
// CTA).  The dot products use four partial sums, so the dependent chain is a
// quarter as long.
__global__ void chol_panel_kernel(double *__restrict__ L, int n, int k0, int kb, const int *__restrict__ info)
{
    if (*info != 0) return;
    __shared__ double lkk[kCholNb][kCholNb + 1];
    __shared__ double inv[kCholNb];
    const int t = threadIdx.x;
    for (int c = 0; c < kCholNb; c++)
        lkk[t][c] = (t < kb && c <= t) ? L[(long long)(k0 + t) * n + k0 + c] : 0.0;
    inv[t] = (t < kb) ? 1.0 / L[(long long)(k0 + t) * n + k0 + t] : 0.0; // one division per CTA lane
    __syncwarp();
    const int i = k0 + kb + blockIdx.x * kCholNb + t;
    if (i >= n) return;
    double *row = L + (long long)i * n + k0;
    double x[kCholNb];
#pragma unroll
    for (int c = 0; c < kCholNb; c++) {
        if (c < kb) {
            double s0 = row[c], s1 = 0.0, s2 = 0.0, s3 = 0.0;
#pragma unroll
            for (int m = 0; m < c; m++) {
                const double p = x[m] * lkk[c][m];
                if ((m & 3) == 0) s0 -= p;
                else if ((m & 3) == 1) s1 -= p;
                else if ((m & 3) == 2) s2 -= p;
                else s3 -= p;
            }
            x[c] = ((s0 + s1) + (s2 + s3)) * inv[c];
            row[c] = x[c];
        } else {
            x[c] = 0.0;
        }
    }
}

// Trailing update: tile (bi, bj), bj <= bi, of the blocks after k0 + kb:
// L_ij -= L_ik L_jk^T (lower triangle only on diagonal tiles).
__global__ void __launch_bounds__(256) chol_update_kernel(double *__restrict__ L, int n, int k0, int kb,
                                                          const int *__restrict__ info)
{
    if (*info != 0) return;
    __shared__ double P[kCholNb][kCholNb + 1], Q[kCholNb][kCholNb + 1];
    // blockIdx.x -> (bi, bj) over the lower triangle of tiles, row by row
    const int t = blockIdx.x;
    int bi = (int)((sqrtf(8.0f * (float)t + 1.0f) - 1.0f) * 0.5f); // then corrected exactly
    while ((bi + 1) * (bi + 2) / 2 <= t) bi++;
    while (bi * (bi + 1) / 2 > t) bi--;
    const int bj = t - bi * (bi + 1) / 2;
    const int r0 = k0 + kb + bi * kCholNb, c0 = k0 + kb + bj * kCholNb;
    for (int e = threadIdx.x; e < kCholNb * kCholNb; e += blockDim.x) {
        const int r = e / kCholNb, m = e % kCholNb;
        P[r][m] = (r0 + r < n && m < kb) ? L[(long long)(r0 + r) * n + k0 + m] : 0.0;
        Q[r][m] = (c0 + r < n && m < kb) ? L[(long long)(c0 + r) * n + k0 + m] : 0.0;
    }
    __syncthreads();
    const int r = threadIdx.x >> 3, cb = (threadIdx.x & 7) * 4;
    const int gi = r0 + r;
    if (gi >= n) return;
#pragma unroll
    for (int u = 0; u < 4; u++) {
        const int c = cb + u, gj = c0 + c;
        if (gj >= n || gj > gi) continue;
        double v = 0.0;
        for (int m = 0; m < kb; m++) v = fma(P[r][m], Q[c][m], v);
        L[(long long)gi * n + gj] -= v;
    }
}

// Packed FP32 rows, and the moment sums in a fixed order (one CTA reduces).
__global__ void chol_finish_kernel(const double *__restrict__ L, int n, float *__restrict__ Lp,
                                   double *__restrict__ aux, const int *__restrict__ info)
{
    __shared__ double red[33];
    if (*info != 0) return;
    // one warp per row
    const int lane = threadIdx.x & 31, warps = (gridDim.x * blockDim.x) >> 5;
    for (int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
        const int off = packed_row_offset(i), len = 4 * (i / 4 + 1);
        for (int j = lane; j < len; j += 32) Lp[off + j] = (j <= i) ? (float)L[(long long)i * n + j] : 0.f;
    }
    if (blockIdx.x == 0) {
        double a = 0.0, b = 0.0;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            a += aux[2 + i];
            b += aux[2 + n + i];
        }
        const double wsw = block_sum(a, red);
        const double wmu = block_sum(b, red);
        if (threadIdx.x == 0) {
            aux[0] = wsw;
            aux[1] = wmu;
        }
    }
}

static cudaError_t launch_cholesky_blocked(const double *A, long long lda, int n, const double *w,
                                           const double *mu, double *L64, float *Lp, float *w32,
                                           double *aux, int *info, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(info, 0, sizeof(int), s);
    if (e != cudaSuccess) return e;
    chol_prep_kernel<<<(n + 7) / 8, 256, 0, s>>>(A, lda, n, w, mu, L64, w32, aux, info);
    for (int k0 = 0; k0 < n; k0 += kCholNb) {
        const int kb = (n - k0 < kCholNb) ? n - k0 : kCholNb;
        chol_diag_kernel<<<1, kCholNb, 0, s>>>(L64, n, k0, kb, info);
        const int rest = n - k0 - kb;
        if (rest > 0) {
            const int mb = (rest + kCholNb - 1) / kCholNb;
            chol_panel_kernel<<<mb, kCholNb, 0, s>>>(L64, n, k0, kb, info);
            chol_update_kernel<<<mb * (mb + 1) / 2, 256, 0, s>>>(L64, n, k0, kb, info);
        }
    }
    chol_finish_kernel<<<(n + 7) / 8, 256, 0, s>>>(L64, n, Lp, aux, info);
    return cudaGetLastError();
}

int cholesky_max_n() { return kCholMaxN; }

// Scratch: aux holds 2 + 2 n doubles (the moments, then the blocked form's
// per-row terms).
cudaError_t launch_cholesky(const double *A, long long lda, int n, const double *w,
                            const double *mu, double *L64, float *Lp, float *w32, double *aux,
                            int *info, cudaStream_t s)
{
    if (n > kCholMaxN) return cudaErrorInvalidValue;
    // RG_CHOLESKY=single|blocked overrides the size rule (for tests)
    const char *sel = getenv("RG_CHOLESKY");
    bool blocked = n > kCholSingleMaxN;
    if (sel && strstr(sel, "single")) blocked = false;
    if (sel && strstr(sel, "blocked")) blocked = true;
    if (blocked) return launch_cholesky_blocked(A, lda, n, w, mu, L64, Lp, w32, aux, info, s);
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
