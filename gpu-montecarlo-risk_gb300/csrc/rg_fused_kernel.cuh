// Plain fused FP32 Monte Carlo kernel, engine (Philox) layout, N <= 64.
//
// Same computation as the reference kernel monte_carlo_kernel
// (src/05-GPU/monte_carlos_cuda.cu:23-72), organised for issue throughput on
// sm_103a:
//
//  * One thread owns one path at a time (grid-stride over paths, grid =
//    SMs x resident CTAs).  Nothing per path reaches HBM unless the caller
//    asks for S or w.R per path.
//  * Row order with packed FP32 pairs.  Row group g (rows 4g..4g+3) needs
//    the normals of quads 0..g; the normals of quad g+1 (one Philox4x32-10
//    block per day, Box-Muller, summed over the H days) are drawn while group
//    g is accumulated, so generator latency hides behind FMAs, and they are
//    kept as float2 pairs.  Each row accumulates (L[i][j], L[i][j+1]) x
//    (z_j, z_j+1) into a float2 with __ffma2_rn (two FMAs per instruction,
//    sm_100+), four rows giving four independent chains; the row value is
//    H mu_i + sum.x + sum.y.  Rows of group g are final at once: compared
//    with -x and folded into S and w.R.
//  * L (packed lower rows), H*mu and w live in the kernel's parameter space,
//    indexed with compile-time offsets: no shared-memory or global loads in
//    the loop.  The packed FFMA2 takes its L pair from registers, so the
//    pairs come through the constant cache (instruction counts: about one
//    load per two FFMA2).  The parameter block is at most 64 packed rows
//    (8.7 KB) plus 2 x 256 B.
//  * Counts: per-thread integers -> warp reduction -> one 64-bit atomic per
//    CTA per counter.
#pragma once
#include <cstring>
#include "rg_internal.cuh"

namespace rg {

static constexpr int kFusedThreads = 256;

template <int NQ>
struct ConstBlock {
    float4 L[packed_len(4 * NQ) / 4]; // packed rows, zero padded
    float4 hmu[NQ];                   // H * mu, FP32 (FP64 product rounded)
    float4 w[NQ];                     // weights (zeros when none)
};

// Normals of quad q of one path, summed over the horizon, divided by
// sqrt(2 ln 2) (the launcher folds that factor into L).
// `second` = false skips the second Box-Muller pair (the last quad when
// N mod 4 is 1 or 2: those normals feed only padding rows).
template <int NQ, bool ONE_DAY>
__device__ __forceinline__ float4 fused_quad_normals(int q, int horizon, uint32_t plo, uint32_t phi,
                                                     const PhiloxKeys &keys, bool second = true)
{
    float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    {
        const uint4 w = rg_philox(make_uint4((uint32_t)q, 0u, plo, phi), keys);
        rg_box_muller_unscaled(w.x, w.y, z.x, z.y);
        if (second) rg_box_muller_unscaled(w.z, w.w, z.z, z.w);
    }
    if (!ONE_DAY) {
        for (int d = 1; d < horizon; d++) {
            const uint4 w = rg_philox(make_uint4((uint32_t)(d * NQ + q), 0u, plo, phi), keys);
            float z0, z1, z2 = 0.f, z3 = 0.f;
            rg_box_muller_unscaled(w.x, w.y, z0, z1);
            if (second) rg_box_muller_unscaled(w.z, w.w, z2, z3);
            z.x += z0;
            z.y += z1;
            z.z += z2;
            z.w += z3;
        }
    }
    return z;
}

// VaR bookkeeping of one path (see PlainArgs): histogram or select pass.
__device__ __forceinline__ void var_path(const PlainArgs &a, float port, unsigned int *shist,
                                         int &n_tail, long long &tail_fx)
{
    const float t = (port - a.sel_lo) * a.sel_inv_w;
    const int b = (t < 0.f) ? -1 : (t >= (float)a.sel_bins ? a.sel_bins : (int)t);
    if (a.var_mode == 2) {
        if (shist) atomicAdd(&shist[b + 1], 1u);
        else atomicAdd(&a.hist[b + 1], 1ull); // kernels without a shared histogram
        return;
    }
    if (b < a.sel_target) {
        n_tail++;
        tail_fx += __float2ll_rn(-port * 4294967296.0f);
    }
    // warp-aggregated append of the candidates
    const bool cand = (b == a.sel_target);
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, cand);
    if (m) {
        const int lane = threadIdx.x & 31;
        const int leader = __ffs(m) - 1;
        unsigned base = 0;
        if (lane == leader) base = atomicAdd(a.cand_count, (unsigned)__popc(m));
        base = __shfl_sync(act, base, leader);
        const unsigned idx = base + __popc(m & ((1u << lane) - 1u));
        if (cand && idx < a.cand_cap) a.cand[idx] = port;
    }
}

// Per-CTA reduction of the counters: warp sums, one 64-bit atomic per CTA
// per counter, and the CTA's histogram merged into the global one.
__device__ __forceinline__ void cta_flush(const PlainArgs &a, int crash, int breach, int n_tail,
                                          long long tail_fx, unsigned long long *sacc,
                                          unsigned int *shist, bool var)
{
    const int tid = threadIdx.x;
    crash = __reduce_add_sync(0xffffffffu, crash);
    breach = __reduce_add_sync(0xffffffffu, breach);
    if (var) {
        n_tail = __reduce_add_sync(0xffffffffu, n_tail);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) tail_fx += __shfl_xor_sync(0xffffffffu, tail_fx, o);
    }
    if ((tid & 31) == 0) {
        atomicAdd(&sacc[0], (unsigned long long)crash);
        atomicAdd(&sacc[1], (unsigned long long)breach);
        if (var) {
            atomicAdd(&sacc[2], (unsigned long long)n_tail);
            atomicAdd(&sacc[3], (unsigned long long)tail_fx);
        }
    }
    __syncthreads();
    if (tid == 0) {
        if (sacc[0]) atomicAdd(&a.counts[0], sacc[0]);
        if (sacc[1]) atomicAdd(&a.counts[1], sacc[1]);
        if (var && a.var_mode == 1) {
            if (sacc[2]) atomicAdd(&a.tail[0], sacc[2]);
            if (sacc[3]) atomicAdd(&a.tail[1], sacc[3]);
        }
    }
    if (shist && a.var_mode == 2)
        for (int t = tid; t < a.sel_bins + 2; t += blockDim.x)
            if (shist[t]) atomicAdd(&a.hist[t], (unsigned long long)shist[t]);
}

// NQ = ceil(N/4) exactly (the launcher dispatches on it), so every row
// group exists; rows >= N occur only in the last group, hold zeros and are
// masked out of S.  ONE_DAY drops the horizon loop for H = 1.  Four CTAs of
// 256 threads per SM (64 registers a thread); with the horizon loop three
// (85 registers: fewer spills, 5 % faster at N = 50, H = 10).  VAR adds the VaR/CVaR
// bookkeeping of var_path (the counting-only form carries none of it).
template <int NQ, bool ONE_DAY, bool VAR>
__global__ void __launch_bounds__(kFusedThreads, ONE_DAY ? 4 : 3) mc_rows_kernel(const PlainArgs a, const ConstBlock<NQ> cb)
{
    __shared__ unsigned long long sacc[4];
    __shared__ unsigned int shist[VAR ? kVarHistBins + 2 : 1];
    const int tid = threadIdx.x;
    if (tid < 4) sacc[tid] = 0ull;
    if (VAR && a.var_mode == 2)
        for (int t = tid; t < a.sel_bins + 2; t += blockDim.x) shist[t] = 0u;
    __syncthreads();
    int n_tail = 0;
    long long tail_fx = 0;

    const int n = a.n;
    // rows of the last group that exist (1..4): the others are skipped
    // (uniform across the grid, so the branches do not diverge)
    const int last_rows = n - 4 * (NQ - 1);
    int crash = 0, breach = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long p = (long long)blockIdx.x * blockDim.x + tid; p < a.n_paths; p += stride) {
        const unsigned long long path = a.path0 + (unsigned long long)p;
        const uint32_t plo = (uint32_t)path, phi = (uint32_t)(path >> 32);
        float2 z2[2 * NQ];
        {
            const float4 z = fused_quad_normals<NQ, ONE_DAY>(0, a.horizon, plo, phi, a.keys, NQ > 1 || last_rows > 2);
            z2[0] = make_float2(z.x, z.y);
            z2[1] = make_float2(z.z, z.w);
        }
        int S = 0;
        float port = 0.f;
#pragma unroll
        for (int g = 0; g < NQ; g++) {
            if (g + 1 < NQ) {
                const float4 z = fused_quad_normals<NQ, ONE_DAY>(g + 1, a.horizon, plo, phi, a.keys,
                                                                 g + 2 < NQ || last_rows > 2);
                z2[2 * g + 2] = make_float2(z.x, z.y);
                z2[2 * g + 3] = make_float2(z.z, z.w);
            }
            float2 acc[4];
#pragma unroll
            for (int e = 0; e < 4; e++) acc[e] = make_float2(0.f, 0.f);
            if (g < NQ - 1) {
#pragma unroll
                for (int q = 0; q <= g; q++) {
#pragma unroll
                    for (int e = 0; e < 4; e++) {
                        const float4 l = cb.L[packed_row_offset(4 * g + e) / 4 + q];
                        acc[e] = __ffma2_rn(make_float2(l.x, l.y), z2[2 * q], acc[e]);
                        acc[e] = __ffma2_rn(make_float2(l.z, l.w), z2[2 * q + 1], acc[e]);
                    }
                }
            } else {
                // last group: rows >= N are padding (same FMA order per row)
#pragma unroll
                for (int e = 0; e < 4; e++) {
                    if (e < last_rows) {
#pragma unroll
                        for (int q = 0; q <= g; q++) {
                            const float4 l = cb.L[packed_row_offset(4 * g + e) / 4 + q];
                            acc[e] = __ffma2_rn(make_float2(l.x, l.y), z2[2 * q], acc[e]);
                            acc[e] = __ffma2_rn(make_float2(l.z, l.w), z2[2 * q + 1], acc[e]);
                        }
                    }
                }
            }
#pragma unroll
            for (int e = 0; e < 4; e++) {
                if (g == NQ - 1 && e >= last_rows) continue;
                const float r = (&cb.hmu[g].x)[e] + (acc[e].x + acc[e].y);
                S += (r < a.neg_x) ? 1 : 0;
                port = fmaf((&cb.w[g].x)[e], r, port);
            }
        }
        crash += (S >= a.k) ? 1 : 0;
        breach += (a.has_w && port < a.port_thr) ? 1 : 0;
        if (a.s_values) a.s_values[p] = S;
        if (a.port_values) a.port_values[p] = port;
        if (VAR) var_path(a, port, shist, n_tail, tail_fx);
    }
    cta_flush(a, crash, breach, n_tail, tail_fx, sacc, VAR ? shist : nullptr, VAR);
}

template <int NQ>
static cudaError_t launch_fused_nq(const PlainArgs &a, const float *Lp_host, const float *hmu,
                                   const float *w, int sm_count, cudaStream_t s)
{
    if (a.n <= 4 * (NQ - 1) || a.n > 4 * NQ) return cudaErrorInvalidValue;
    ConstBlock<NQ> cb;
    memset(&cb, 0, sizeof(cb));
    memcpy(cb.L, Lp_host, sizeof(float) * (size_t)packed_len(a.n));
    {
        // the kernel draws z / sqrt(2 ln 2) (rg_box_muller_unscaled): R = H mu + (s L) z with
        // s = sqrt(2 ln 2), times sqrt(H) with one N(0, 1) draw per asset (aggregated)
        const float sh = (float)((double)kBmScale * (a.aggregated ? std::sqrt((double)a.horizon) : 1.0));
        float *Lf = reinterpret_cast<float *>(cb.L);
        for (int i = 0; i < packed_len(a.n); i++) Lf[i] *= sh;
    }
    memcpy(cb.hmu, hmu, sizeof(float) * (size_t)a.n);
    memcpy(cb.w, w, sizeof(float) * (size_t)a.n);
    const bool one_day = (a.horizon == 1 || a.aggregated);
    auto kern = (a.var_mode != 0) ? (one_day ? mc_rows_kernel<NQ, true, true> : mc_rows_kernel<NQ, false, true>)
                : one_day ? mc_rows_kernel<NQ, true, false> : mc_rows_kernel<NQ, false, false>;
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, kFusedThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    long long want = (a.n_paths + kFusedThreads - 1) / kFusedThreads;
    long long grid = (long long)sm_count * per_sm;
    if (want < grid) grid = want;
    if (grid < 1) grid = 1;
    kern<<<(unsigned)grid, kFusedThreads, 0, s>>>(a, cb);
    return cudaGetLastError();
}

} // namespace rg
