// Plain fused FP32 Monte Carlo kernel for N <= 64 assets.
//
// Replaces the reference kernel monte_carlo_kernel
// (src/05-GPU/monte_carlos_cuda.cu:23-72).  One thread owns one path at a
// time (grid sized to fill every SM; grid-stride over paths in the Philox
// layout, a contiguous run of paths per thread in the XORWOW layout):
//   1. normals in registers: Philox4x32-10 + Box-Muller (engine layout) or
//      the reference's own cuRAND XORWOW stream (curand_init(seed, path, 0)
//      + curand_normal_double, rounded to FP32), summed over H days;
//   2. R_i = H mu_i + sum_{j<=i} L_ij Zsum_j in FP32 with L's packed rows
//      staged once per CTA in shared memory and read as broadcast float4;
//   3. S = #{R_i < -x}, portfolio return w.R, crash (S >= k) and breach
//      (w.R < threshold) flags;
//   4. per-thread integer counts -> warp reduction -> one 64-bit atomic per
//      CTA per counter.
// Nothing per path reaches HBM unless the caller asks for S or w.R per path
// (parity tests; the reference always writes S, .cu:67).
//
// The asset loops are fully unrolled for a compile-time bound NP (16, 32 or
// 64) so that Z lives in registers; the runtime N <= NP is handled by
// uniform early exits, so no arithmetic is spent on padding rows.
#pragma once
#include <curand_kernel.h>
#include "rg_internal.cuh"

namespace rg {

static constexpr int kPlainThreads = 256;

template <int NP, int RNG>
__global__ void __launch_bounds__(kPlainThreads, 2) mc_plain_small_kernel(const PlainArgs a)
{
    constexpr int NQ = NP / 4;
    constexpr int PACK4 = packed_len(NP) / 4;
    __shared__ float4 sL[PACK4];
    __shared__ float shmu[NP];
    __shared__ float sw[NP];
    __shared__ unsigned long long sacc[2];

    const int n = a.n;
    const int tid = threadIdx.x;
    const int have4 = packed_len(n) / 4;
    for (int t = tid; t < PACK4; t += blockDim.x)
        sL[t] = (t < have4) ? a.Lp[t] : make_float4(0.f, 0.f, 0.f, 0.f);
    for (int t = tid; t < NP; t += blockDim.x) {
        shmu[t] = (t < n) ? (float)((double)a.horizon * a.mu64[t]) : 0.f;
        sw[t] = (t < n && a.has_w) ? a.w[t] : 0.f;
    }
    if (tid < 2) sacc[tid] = 0ull;
    __syncthreads();

    const int nq = (n + 3) >> 2;
    int crash = 0, breach = 0;
    // Philox: grid-stride over paths.  XORWOW: each thread walks a
    // contiguous run of paths, so the cuRAND state of path p + 1 (the
    // seeded state advanced by p + 1 subsequences) comes from the saved
    // state of path p by one cuRAND skipahead_sequence(1) instead of a full
    // curand_init(seed, p + 1, 0), whose skip-ahead costs about one matrix
    // product per base-4 digit of the path index.
    const long long nthreads = (long long)gridDim.x * blockDim.x;
    const long long gtid = (long long)blockIdx.x * blockDim.x + tid;
    long long p_begin = gtid, p_end = a.n_paths, p_step = nthreads;
    if (RNG != RG_RNG_PHILOX) {
        const long long chunk = (a.n_paths + nthreads - 1) / nthreads;
        p_begin = gtid * chunk;
        p_end = p_begin + chunk < a.n_paths ? p_begin + chunk : a.n_paths;
        p_step = 1;
    }
    curandStateXORWOW_t next_state;
    if (RNG != RG_RNG_PHILOX && p_begin < p_end)
        curand_init(a.seed, a.path0 + (unsigned long long)p_begin, 0ull, &next_state);
    for (long long p = p_begin; p < p_end; p += p_step) {
        const unsigned long long path = a.path0 + (unsigned long long)p;
        float z[NP];
#pragma unroll
        for (int j = 0; j < NP; j++) z[j] = 0.f;

        if (RNG == RG_RNG_PHILOX) {
            for (int d = 0; d < a.horizon; d++) {
#pragma unroll
                for (int q = 0; q < NQ; q++) {
                    if (q < nq) {
                        const uint4 c = make_uint4((uint32_t)(d * nq + q), 0u, (uint32_t)path,
                                                   (uint32_t)(path >> 32));
                        const uint4 r = rg_philox(c, a.keys);
                        float z0, z1, z2, z3;
                        rg_box_muller(r.x, r.y, z0, z1);
                        rg_box_muller(r.z, r.w, z2, z3);
                        z[4 * q + 0] += z0;
                        z[4 * q + 1] += z1;
                        z[4 * q + 2] += z2;
                        z[4 * q + 3] += z3;
                    }
                }
            }
        } else {
            // this path's state as curand_init(seed, path, 0) leaves it
            curandStateXORWOW_t st = next_state;
            if (p + 1 < p_end) skipahead_sequence(1ull, &next_state);
            for (int d = 0; d < a.horizon; d++) {
#pragma unroll
                for (int j = 0; j < NP; j++)
                    if (j < n) z[j] += (float)curand_normal_double(&st);
            }
        }

        int S = 0;
        float port = 0.f;
#pragma unroll
        for (int i = 0; i < NP; i++) {
            if (i < n) {
                const float4 *row = sL + packed_row_offset(i) / 4;
                float acc0 = shmu[i], acc1 = 0.f;
#pragma unroll
                for (int q = 0; q <= i / 4; q++) {
                    const float4 l = row[q];
                    if (q & 1) {
                        acc1 = fmaf(l.x, z[4 * q + 0], acc1);
                        acc1 = fmaf(l.y, z[4 * q + 1], acc1);
                        acc1 = fmaf(l.z, z[4 * q + 2], acc1);
                        acc1 = fmaf(l.w, z[4 * q + 3], acc1);
                    } else {
                        acc0 = fmaf(l.x, z[4 * q + 0], acc0);
                        acc0 = fmaf(l.y, z[4 * q + 1], acc0);
                        acc0 = fmaf(l.z, z[4 * q + 2], acc0);
                        acc0 = fmaf(l.w, z[4 * q + 3], acc0);
                    }
                }
                const float r = acc0 + acc1;
                S += (r < a.neg_x) ? 1 : 0;
                port = fmaf(sw[i], r, port);
            }
        }
        crash += (S >= a.k) ? 1 : 0;
        breach += (a.has_w && port < a.port_thr) ? 1 : 0;
        if (a.s_values) a.s_values[p] = S;
        if (a.port_values) a.port_values[p] = port;
    }

    crash = __reduce_add_sync(0xffffffffu, crash);
    breach = __reduce_add_sync(0xffffffffu, breach);
    if ((tid & 31) == 0) {
        atomicAdd(&sacc[0], (unsigned long long)crash);
        atomicAdd(&sacc[1], (unsigned long long)breach);
    }
    __syncthreads();
    if (tid == 0) {
        if (sacc[0]) atomicAdd(&a.counts[0], sacc[0]);
        if (sacc[1]) atomicAdd(&a.counts[1], sacc[1]);
    }
}

template <int NP, int RNG>
static cudaError_t launch_np(const PlainArgs &a, int sm_count, cudaStream_t s)
{
    auto kern = mc_plain_small_kernel<NP, RNG>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kPlainThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    long long want = (a.n_paths + kPlainThreads - 1) / kPlainThreads;
    long long grid = (long long)sm_count * per_sm;
    if (want < grid) grid = want;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, kPlainThreads, 0, s>>>(a);
    return cudaGetLastError();
}

} // namespace rg
