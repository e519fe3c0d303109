// Plain fused FP32 Monte Carlo kernel for any asset count (the general-N
// counterpart of the N <= 64 kernel; the reference caps N at 64,
// src/05-GPU/monte_carlos_cuda.cu:34,78-81).
//
// A CTA owns a tile of 64 paths at a time (grid-stride over tiles):
//  1. Normals.  The 256 threads draw the tile's normals (Philox4x32-10 in
//     the engine layout, Box-Muller, summed over the H days -- or one
//     N(0, H) draw per asset in the aggregated mode) into shared memory,
//     Zs[k][p] (asset-major rows of 64 paths, FP32).
//  2. Contraction R = H mu + L Z as an FP32 GEMM over 128-asset column
//     blocks: each thread holds a 4-path x 8-asset register tile, reads
//     Z (float4, 4 paths) and L^T (two float4, 8 assets) from shared memory
//     and accumulates with packed __ffma2_rn; the K loop of column block c
//     stops at 128 (c+1) because L is lower triangular.  L^T slices (8 x 128)
//     are staged by the CTA, double buffered with cp.async.
//  3. Per column block each thread folds its 4 x 8 returns into per-path
//     partial crash counts and w.R partial sums in shared memory; the 16
//     asset groups are summed in a fixed order (deterministic), and after
//     the last block one thread per path forms S, w.R, the crash and breach
//     flags and the VaR bookkeeping.
// Shared memory: 4 * 64 * Kpad bytes for Z (155 KB at N = 600) + 8 KB of L
// staging + 8 KB of partials (+ 16 KB of VaR histogram): one CTA per SM,
// N <= 768.
#include <cstring>
#include "rg_fused_kernel.cuh"

namespace rg {

static constexpr int kTP = 64;        // paths per tile
static constexpr int kTN = 128;       // assets per column block
static constexpr int kTK = 8;         // K slice staged per step
static constexpr int kTiledThreads = 256;

struct TiledArgs {
    PlainArgs a;          // counters, thresholds, Philox keys, VaR fields
    const float *Lt;      // [kpad][npad] L^T, FP32, zero padded
    int kpad;             // N rounded up to kTK
    int npad;             // N rounded up to kTN
    int aggregated;       // 1: one N(0, H) draw per asset (sqrt(H) z)
    float sqrt_h;
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

template <bool VAR>
__global__ void __launch_bounds__(kTiledThreads, 1) mc_tiled_kernel(const TiledArgs t)
{
    extern __shared__ __align__(16) float smem[];
    const PlainArgs &a = t.a;
    const int kpad = t.kpad;
    float *Zs = smem;                                  // [kpad][kTP]
    float *Ls = Zs + (size_t)kpad * kTP;               // [2][kTK][kTN]
    int *partS = (int *)(Ls + 2 * kTK * kTN);          // [16][kTP]
    float *partP = (float *)(partS + 16 * kTP);        // [16][kTP]
    __shared__ int totS[kTP];
    __shared__ float totP[kTP];
    __shared__ unsigned long long sacc[4];
    __shared__ unsigned int shist[VAR ? kVarHistBins + 2 : 1];

    const int tid = threadIdx.x;
    if (tid < 4) sacc[tid] = 0ull;
    if (VAR && a.var_mode == 2)
        for (int i = tid; i < a.sel_bins + 2; i += blockDim.x) shist[i] = 0u;
    int crash = 0, breach = 0, n_tail = 0;
    long long tail_fx = 0;
    const int n = a.n;
    const int nq = (n + 3) >> 2;
    const int ncb = (n + kTN - 1) / kTN;
    // register tile: paths 4*pg .. 4*pg+3, assets 8*ag .. 8*ag+7 of a block
    const int pg = tid & 15, ag = tid >> 4;
    const long long ntiles = (a.n_paths + kTP - 1) / kTP;

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long p0 = tile * kTP;
        // ---- 1. normals into Zs[k][p]
        {
            const int p = tid & (kTP - 1), r = tid >> 6; // 4 threads per path
            const unsigned long long path = a.path0 + (unsigned long long)(p0 + p);
            const uint32_t plo = (uint32_t)path, phi = (uint32_t)(path >> 32);
            for (int q = r; q < kpad / 4; q += 4) {
                float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
                if (q < nq) {
                    const int days = t.aggregated ? 1 : a.horizon;
                    for (int d = 0; d < days; d++) {
                        const uint4 wv = rg_philox(make_uint4((uint32_t)(d * nq + q), 0u, plo, phi), a.keys);
                        float z0, z1, z2, z3;
                        rg_box_muller(wv.x, wv.y, z0, z1);
                        rg_box_muller(wv.z, wv.w, z2, z3);
                        z.x += z0;
                        z.y += z1;
                        z.z += z2;
                        z.w += z3;
                    }
                    if (t.aggregated) {
                        z.x *= t.sqrt_h;
                        z.y *= t.sqrt_h;
                        z.z *= t.sqrt_h;
                        z.w *= t.sqrt_h;
                    }
                }
                Zs[(4 * q + 0) * kTP + p] = z.x;
                Zs[(4 * q + 1) * kTP + p] = z.y;
                Zs[(4 * q + 2) * kTP + p] = z.z;
                Zs[(4 * q + 3) * kTP + p] = z.w;
            }
        }
        if (tid < kTP) {
            totS[tid] = 0;
            totP[tid] = 0.f;
        }
        __syncthreads();

        // ---- 2./3. column blocks
        for (int cb = 0; cb < ncb; cb++) {
            const int c0 = cb * kTN;
            const int kmax = min(kpad, c0 + kTN);
            float2 acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = make_float2(0.f, 0.f);
            // stage slice 0
            {
                const int kk = tid >> 5, c4 = tid & 31; // 8 rows x 32 float4
                cp_async16(&Ls[kk * kTN + 4 * c4], &t.Lt[(size_t)kk * t.npad + c0 + 4 * c4]);
                cp_async_commit();
            }
            int buf = 0;
            for (int k0 = 0; k0 < kmax; k0 += kTK) {
                cp_async_wait_all();
                __syncthreads();
                if (k0 + kTK < kmax) {
                    const int kk = tid >> 5, c4 = tid & 31;
                    cp_async16(&Ls[(buf ^ 1) * kTK * kTN + kk * kTN + 4 * c4],
                               &t.Lt[(size_t)(k0 + kTK + kk) * t.npad + c0 + 4 * c4]);
                    cp_async_commit();
                }
                const float *Lb = Ls + buf * kTK * kTN;
#pragma unroll
                for (int kk = 0; kk < kTK; kk++) {
                    const float4 z = *reinterpret_cast<const float4 *>(&Zs[(k0 + kk) * kTP + 4 * pg]);
                    const float4 l0 = *reinterpret_cast<const float4 *>(&Lb[kk * kTN + 8 * ag]);
                    const float4 l1 = *reinterpret_cast<const float4 *>(&Lb[kk * kTN + 8 * ag + 4]);
                    const float zz[4] = {z.x, z.y, z.z, z.w};
#pragma unroll
                    for (int i = 0; i < 4; i++) {
                        const float2 zi = make_float2(zz[i], zz[i]);
                        acc[i][0] = __ffma2_rn(make_float2(l0.x, l0.y), zi, acc[i][0]);
                        acc[i][1] = __ffma2_rn(make_float2(l0.z, l0.w), zi, acc[i][1]);
                        acc[i][2] = __ffma2_rn(make_float2(l1.x, l1.y), zi, acc[i][2]);
                        acc[i][3] = __ffma2_rn(make_float2(l1.z, l1.w), zi, acc[i][3]);
                    }
                }
                buf ^= 1;
            }
            // epilogue of the block: partial S and w.R per path
            float hm[8], wt[8];
#pragma unroll
            for (int j = 0; j < 8; j++) {
                const int c = c0 + 8 * ag + j;
                hm[j] = (c < n) ? (float)((double)a.horizon * a.mu64[c]) : 0.f;
                wt[j] = (c < n) ? a.w[c] : 0.f;
            }
#pragma unroll
            for (int i = 0; i < 4; i++) {
                int s = 0;
                float pw = 0.f;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int a0 = c0 + 8 * ag + 2 * j;
                    const float r0 = hm[2 * j] + acc[i][j].x;
                    const float r1 = hm[2 * j + 1] + acc[i][j].y;
                    s += (a0 < n && r0 < a.neg_x) ? 1 : 0;
                    s += (a0 + 1 < n && r1 < a.neg_x) ? 1 : 0;
                    pw = fmaf(wt[2 * j], r0, pw);
                    pw = fmaf(wt[2 * j + 1], r1, pw);
                }
                partS[ag * kTP + 4 * pg + i] = s;
                partP[ag * kTP + 4 * pg + i] = pw;
            }
            __syncthreads();
            if (tid < kTP) {
                int s = totS[tid];
                float pw = totP[tid];
#pragma unroll
                for (int g = 0; g < 16; g++) {
                    s += partS[g * kTP + tid];
                    pw += partP[g * kTP + tid];
                }
                totS[tid] = s;
                totP[tid] = pw;
            }
            // partS/partP and Ls are rewritten only after the next barrier
        }
        __syncthreads();
        // ---- per-path results (warps 0 and 1)
        if (tid < kTP) {
            const long long p = p0 + tid;
            if (p < a.n_paths) {
                const int S = totS[tid];
                const float port = totP[tid];
                crash += (S >= a.k) ? 1 : 0;
                breach += (a.has_w && port < a.port_thr) ? 1 : 0;
                if (a.s_values) a.s_values[p] = S;
                if (a.port_values) a.port_values[p] = port;
                if (VAR) var_path(a, port, shist, n_tail, tail_fx);
            }
        }
        __syncthreads();
    }
    cta_flush(a, crash, breach, n_tail, tail_fx, sacc, VAR ? shist : nullptr, VAR);
}

int tiled_max_n() { return 768; }

size_t tiled_smem_bytes(int n)
{
    const int kpad = (n + kTK - 1) / kTK * kTK;
    return sizeof(float) * ((size_t)kpad * kTP + 2 * kTK * kTN + 2 * 16 * kTP);
}

int tiled_npad(int n) { return (n + kTN - 1) / kTN * kTN; }
int tiled_kpad(int n) { return (n + kTK - 1) / kTK * kTK; }

cudaError_t launch_tiled(const PlainArgs &a, const float *Lt, bool aggregated, int sm_count,
                         cudaStream_t s)
{
    if (a.n > tiled_max_n()) return cudaErrorInvalidValue;
    TiledArgs t;
    memset(&t, 0, sizeof(t));
    t.a = a;
    t.Lt = Lt;
    t.kpad = tiled_kpad(a.n);
    t.npad = tiled_npad(a.n);
    t.aggregated = aggregated ? 1 : 0;
    t.sqrt_h = sqrtf((float)a.horizon);
    const size_t smem = tiled_smem_bytes(a.n);
    auto kern = (a.var_mode != 0) ? mc_tiled_kernel<true> : mc_tiled_kernel<false>;
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    long long tiles = (a.n_paths + kTP - 1) / kTP;
    long long grid = sm_count;
    if (tiles < grid) grid = tiles;
    kern<<<(unsigned)grid, kTiledThreads, smem, s>>>(t);
    return cudaGetLastError();
}

// L^T (FP32, [kpad][npad], zero padded), H-independent; and weights padded.
__global__ void build_lt_kernel(const double *L, int n, int kpad, int npad, float *Lt)
{
    const long long total = (long long)kpad * npad;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int k = (int)(idx / npad), c = (int)(idx % npad);
        float v = 0.f;
        if (k < n && c < n && k <= c) v = (float)L[(long long)c * n + k];
        Lt[idx] = v;
    }
}

cudaError_t launch_build_lt(const double *L64, int n, float *Lt, cudaStream_t s)
{
    const int kpad = tiled_kpad(n), npad = tiled_npad(n);
    build_lt_kernel<<<256, 256, 0, s>>>(L64, n, kpad, npad, Lt);
    return cudaGetLastError();
}

} // namespace rg
