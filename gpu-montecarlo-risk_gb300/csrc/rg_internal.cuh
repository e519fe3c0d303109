// Internal declarations shared by the engine's translation units.
//
// Device helpers:
//   rg_philox       Philox4x32-10 (Salmon et al., SC'11): 10 rounds of two
//                   32x32->64 multiplies with the published multipliers and
//                   Weyl key increments.  Round keys are precomputed on the
//                   host (they depend only on the seed).
//   rg_box_muller   Box-Muller (Box & Muller 1958) on two 32-bit words.
//                   The top 23 bits of a word w form f = 1 + (w >> 9) 2^-23 in
//                   [1, 2) by setting the exponent bits (no int->float
//                   conversion); u_a = 2 - f in (0, 1], t = 2 pi f_b in
//                   [2 pi, 4 pi) (a uniform angle), r = sqrt(-2 ln u_a),
//                   (z0, z1) = (r cos t, r sin t), using the hardware
//                   approximate lg2/sqrt/sin/cos (PTX *.approx).  The
//                   smallest u_a is 2^-23, so |z| <= sqrt(46 ln 2) = 5.65.
#pragma once

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "riskgpu.h"

namespace rg {

// ---------------------------------------------------------------- device
struct PhiloxKeys {
    uint32_t k0[10];
    uint32_t k1[10];
};

inline PhiloxKeys philox_round_keys(uint64_t seed)
{
    PhiloxKeys k;
    uint32_t a = (uint32_t)seed, b = (uint32_t)(seed >> 32);
    for (int r = 0; r < 10; r++) {
        k.k0[r] = a;
        k.k1[r] = b;
        a += 0x9E3779B9u;
        b += 0xBB67AE85u;
    }
    return k;
}

__device__ __forceinline__ uint4 rg_philox(uint4 c, const PhiloxKeys &k)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * c.x;
        const uint64_t p1 = (uint64_t)0xCD9E8D57u * c.z;
        const uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        const uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        c = make_uint4(hi1 ^ c.y ^ k.k0[r], lo1, hi0 ^ c.w ^ k.k1[r], lo0);
    }
    return c;
}

// Two independent Philox4x32-10 blocks, rounds interleaved (the same words
// as two rg_philox calls; more independent work per thread where few warps
// share an SM).
__device__ __forceinline__ void rg_philox2(uint4 &a, uint4 &b, const PhiloxKeys &k)
{
#pragma unroll
    for (int r = 0; r < 10; r++) {
        const uint64_t p0 = (uint64_t)0xD2511F53u * a.x, p1 = (uint64_t)0xCD9E8D57u * a.z;
        const uint64_t q0 = (uint64_t)0xD2511F53u * b.x, q1 = (uint64_t)0xCD9E8D57u * b.z;
        a = make_uint4((uint32_t)(p1 >> 32) ^ a.y ^ k.k0[r], (uint32_t)p1, (uint32_t)(p0 >> 32) ^ a.w ^ k.k1[r],
                       (uint32_t)p0);
        b = make_uint4((uint32_t)(q1 >> 32) ^ b.y ^ k.k0[r], (uint32_t)q1, (uint32_t)(q0 >> 32) ^ b.w ^ k.k1[r],
                       (uint32_t)q0);
    }
}

__device__ __forceinline__ float rg_lg2_approx(float x)
{
    float y;
    asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rg_sqrt_approx(float x)
{
    float y;
    asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rg_sin_approx(float x)
{
    float y;
    asm("sin.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}
__device__ __forceinline__ float rg_cos_approx(float x)
{
    float y;
    asm("cos.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    return y;
}

// 1 + (w >> 9) 2^-23, exactly, in [1, 2)
__device__ __forceinline__ float rg_one_to_two(uint32_t w)
{
    return __uint_as_float(0x3f800000u | (w >> 9));
}

__device__ __forceinline__ void rg_box_muller(uint32_t a, uint32_t b, float &z0, float &z1)
{
    const float ua = 2.0f - rg_one_to_two(a);          // (0, 1]
    // -2 ln(u) = -2 ln(2) log2(u)
    const float r = rg_sqrt_approx(-1.3862943611198906f * rg_lg2_approx(ua));
    const float t = 6.283185307179586f * rg_one_to_two(b); // [2 pi, 4 pi)
    z0 = r * rg_cos_approx(t);
    z1 = r * rg_sin_approx(t);
}

// sqrt(2 ln 2): r = sqrt(-2 ln u) = kBmScale sqrt(-log2 u).
static constexpr float kBmScale = 1.1774100225154747f;

// Box-Muller as above without the factor sqrt(2 ln 2) of r: returns
// (z0, z1) / sqrt(2 ln 2), one multiply fewer a pair.  For callers that sum
// several draws and scale the sum once.
__device__ __forceinline__ void rg_box_muller_unscaled(uint32_t a, uint32_t b, float &z0, float &z1)
{
    const float ua = 2.0f - rg_one_to_two(a);          // (0, 1]
    const float r = rg_sqrt_approx(-rg_lg2_approx(ua));
    const float t = 6.283185307179586f * rg_one_to_two(b); // [2 pi, 4 pi)
    z0 = r * rg_cos_approx(t);
    z1 = r * rg_sin_approx(t);
}

// Packed FP32 lower-triangular rows: row i holds L[i][0..i] zero-padded to
// a multiple of 4 floats, so every row starts on a 16-byte boundary.
// offset(i) = sum_{r<i} 4 ceil((r+1)/4) = 4 (a+1)(2a+b) for i = 4a+b.
__host__ __device__ constexpr int packed_row_offset(int i)
{
    return 4 * (i / 4 + 1) * (2 * (i / 4) + (i % 4));
}
__host__ __device__ constexpr int packed_len(int n) { return packed_row_offset(n); }

// ---------------------------------------------------------------- host
struct Portfolio {
    int n = 0;
    int has_w = 0;
    int device = 0;
    void *d_block = nullptr;   // one allocation holding every device buffer below
    double *d_L64 = nullptr;   // n x n row-major, zero upper
    double *d_mu64 = nullptr;  // n
    float *d_Lp = nullptr;     // packed rows (packed_len(n) floats)
    float *d_Lt = nullptr;     // L^T FP32 [tiled_kpad(n)][tiled_npad(n)], zero padded
    unsigned char *d_tc[2] = {nullptr, nullptr}; // tensor-core tiles (FP16, BF16), N <= tc_max_n()
    unsigned int *d_err = nullptr; // error word of the tensor-core kernel
    float *d_w32 = nullptr;    // n (zeros when no weights)
    double *d_aux = nullptr;   // [2 + 2n]: w^T Sigma w, w.mu, then factorisation scratch
    int *d_info = nullptr;
    double wsw = 0.0, wmu = 0.0;
    float ms_chol = 0.f;
    // host copies for kernels that take the factor by value
    std::vector<float> h_Lp;   // packed rows, FP32
    std::vector<double> h_mu;  // daily means, FP64
    std::vector<float> h_w;    // weights, FP32 (zeros when none)
};

// Arguments of the fused counting kernels.
struct PlainArgs {
    const float4 *Lp;
    const double *mu64;
    const float *w;
    int n;
    int horizon;
    long long n_paths;
    unsigned long long path0;
    unsigned long long seed;
    PhiloxKeys keys;
    float neg_x;
    float port_thr;
    int k;
    int has_w;
    int aggregated;            // draw mode RG_DRAWS_AGGREGATED
    int *s_values;
    float *port_values;
    unsigned long long *counts; // [2]
    // VaR / CVaR passes (kernels instantiated with VaR support only).
    // Every path's portfolio return w.R falls in bin
    //   b = floor((w.R - sel_lo) * sel_inv_w), clamped to [-1, sel_bins].
    // var_mode 1 (select): b < sel_target -> tail (count, fixed-point loss
    //   sum); b == sel_target -> candidate appended to cand[].
    // var_mode 2 (histogram): counts per bin into hist[sel_bins + 2].
    int var_mode;
    int sel_bins;
    int sel_target;
    float sel_lo;
    float sel_inv_w;
    float *cand;
    unsigned int *cand_count;
    unsigned int cand_cap;
    unsigned long long *tail;   // [0] tail paths, [1] sum of -w.R * 2^32 (int64 bits)
    unsigned long long *hist;   // [sel_bins + 2]
    unsigned int *err;          // device error word of the tensor-core kernel (bounded waits)
};

// Shared-memory histogram size of the VaR pass: bins plus under/overflow.
static constexpr int kVarHistBins = 4096;

// Launchers.  Return cudaSuccess or the launch error.
// rg_mc_plain.cu / rg_mc_xorwow.cu: row-order kernel, L staged in shared
// memory; both normal layouts.
cudaError_t launch_plain_small(const PlainArgs &a, int rng, int sm_count, cudaStream_t s);
int plain_small_max_n();
// rg_mc_tiled.cu: general-N tiled kernel (Philox layout).
cudaError_t launch_tiled(const PlainArgs &a, const float *Lt, bool aggregated, int sm_count,
                         cudaStream_t s);
cudaError_t launch_build_lt(const double *L64, int n, float *Lt, cudaStream_t s);
int tiled_max_n();
int tiled_npad(int n);
int tiled_kpad(int n);
// rg_mc_tc.cu: tcgen05 precision form (Philox layout), N <= tc_max_n().
cudaError_t launch_tc(const PlainArgs &a, const unsigned char *tiles, int bf16, bool aggregated, double wmu,
                      unsigned int *err, bool inject_stall, int sm_count, cudaStream_t s);
cudaError_t launch_build_tc_tiles(const double *L64, const float *w32, int n, int bf16, unsigned char *tiles,
                                  cudaStream_t s);
int tc_max_n();
size_t tc_tile_bytes(int n);
// batches of (portfolio, query) items in one persistent launch
void tc_fill_batch_item(void *item_out, const PlainArgs &a, const unsigned char *tiles, int bf16,
                        bool aggregated, double wmu, long long tile_begin);
size_t tc_item_bytes();
long long tc_tiles_of(long long n_paths, int paths_per_tile);
int tc_batch_paths(int n_mt_max);
int tc_row_tiles_of(int n);
int tc_k_tiles_of(int n);
cudaError_t launch_tc_batch(const void *d_items, int n_items, long long total_tiles, int unit_tiles,
                            unsigned int *work, unsigned int *err, int n_kt_max, int n_mt_max, int grid,
                            cudaStream_t s, const long long *dyn = nullptr);
int tc_max_k_tiles();
cudaError_t tc_batch_prepare();
int tc_batch_occupancy(int n_mt_max);
// rg_mc_fused.cu: N <= 64 kernel, L in parameter space; Philox only.
cudaError_t launch_fused(const PlainArgs &a, const float *Lp_host, const float *hmu, const float *w,
                         int sm_count, cudaStream_t s);
int fused_max_n();

// Cholesky (rg_cholesky.cu): factor, pack and portfolio moments.
cudaError_t launch_cholesky(const double *A, long long lda, int n, const double *w,
                            const double *mu, double *L64, float *Lp, float *w32, double *aux,
                            int *info, cudaStream_t s);
int cholesky_max_n();

// Error helpers (rg_capi.cu).
int set_error(int status, const char *fmt, ...);

} // namespace rg
