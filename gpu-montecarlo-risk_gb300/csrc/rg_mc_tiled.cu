// Plain fused FP32 Monte Carlo kernels for any asset count (the general-N
// counterpart of the N <= 64 kernel; the reference caps N at 64,
// src/05-GPU/monte_carlos_cuda.cu:34,78-81).  Three forms, each described
// at its definition: the pipelined mc_tiled_pipe_kernel (default), the
// phase-serial mc_tiled_kernel it is built from (RG_PLAIN_KERNEL=serial) and
// the warp-specialised mc_tiled_ws_kernel (RG_PLAIN_KERNEL=ws).  At N = 600,
// H = 10, 1e7 paths: 116.8, 136.6 and 170 ms with daily draws; 86.5, 94.1
// and 149 ms with aggregated draws.
//
// Phase-serial form: a CTA owns a tile of 64 paths at a time (grid-stride
// over tiles):
//  1. Normals.  The 256 threads draw the tile's normals (Philox4x32-10 in
//     the engine layout, Box-Muller, summed over the H days -- or one
//     N(0, H) draw per asset in the aggregated mode) into shared memory,
//     Zs[k][p] (asset-major rows of 64 paths, FP32), two quads per thread
//     at a time with their Philox rounds interleaved.
//  2. Contraction R = H mu + L Z as an FP32 GEMM over 128-asset column
//     blocks: each thread holds a 4-path x 8-asset register tile, reads
//     Z (float4, 4 paths) and L^T (two float4, 8 assets) from shared memory
//     and accumulates with packed __ffma2_rn.  L is lower triangular, so
//     warp w (assets c0 + 16w .. c0 + 16w + 15) stops its multiply-adds at
//     c0 + 16(w + 1).  L^T slices (KT x 128, KT = 16 where shared memory
//     allows, else 8) are staged by the CTA, double buffered with cp.async.
//  3. Per column block each thread folds its 4 x 8 returns into per-path
//     partial crash counts and w.R partial sums in shared memory; the 16
//     asset groups are summed in a fixed order (deterministic), and after
//     the last block one thread per path forms S, w.R, the crash and breach
//     flags and the VaR bookkeeping.
// Shared memory: 256 x Kpad bytes for Z (156 KB at N = 600) + 2 x KT x 512
// bytes of L staging + 8 KB of partials (+ 16 KB of VaR histogram): one CTA
// per SM, N <= 768.  Generation and the GEMM take turns on 8 warps per SM.
#include <cstdlib>
#include <cstring>
#include "rg_fused_kernel.cuh"

namespace rg {

static constexpr int kTP = 64;        // paths per tile
static constexpr int kTiledMaxN = 768; // assets (K padded to 32, columns to 256)
static constexpr int kTN = 128;       // assets per column block
static constexpr int kTK = 8;         // K slice staged per step (warp-specialised form)
static constexpr int kTiledThreads = 256;

struct TiledArgs {
    PlainArgs a;          // counters, thresholds, Philox keys, VaR fields
    const float *Lt;      // [kpad][npad] L^T, FP32, zero padded
    int kpad;             // N rounded up to 32 (tiled_kpad)
    int npad;             // N rounded up to 256 (a multiple of both column-block widths)
    int aggregated;       // 1: one N(0, H) draw per asset (sqrt(H) z)
    float zscale;         // factor of each summed normal: sqrt(2 ln 2) (the draws are unscaled), x sqrt(H) aggregated
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem)
{
    const unsigned s = (unsigned)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(s), "l"(gmem));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;"); }
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_group 0;" ::: "memory"); }

// KT: rows of L^T staged per step (16 where shared memory allows, else 8).
// THREADS: 256 (8 warps, 128-asset column blocks).  The kernel is also
// correct with 512 (16 warps, 256-asset blocks), which measured slower at
// N = 600, H = 10 (139 against 137 ms per 1e7 paths; aggregated draws 99
// against 94 ms), so the launcher uses 256.
template <bool VAR, int KT, int THREADS>
__global__ void __launch_bounds__(THREADS, 1) mc_tiled_kernel(const TiledArgs t)
{
    constexpr int TN = THREADS / 2;   // assets per column block (8 per thread column)
    constexpr int NAG = THREADS / 16; // asset groups of 8
    constexpr int R = THREADS / 64;   // threads per path in the normal draws
    extern __shared__ __align__(16) float smem[];
    const PlainArgs &a = t.a;
    const int kpad = t.kpad;
    float *Zs = smem;                                  // [kpad][kTP]
    float *Ls = Zs + (size_t)kpad * kTP;               // [2][KT][TN]
    int *partS = (int *)(Ls + 2 * KT * TN);            // [NAG][kTP]
    float *partP = (float *)(partS + NAG * kTP);       // [NAG][kTP]
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
    const int ncb = (n + TN - 1) / TN;
    // register tile: paths 4*pg .. 4*pg+3, assets 8*ag .. 8*ag+7 of a block
    const int pg = tid & 15, ag = tid >> 4;
    const long long ntiles = (a.n_paths + kTP - 1) / kTP;

    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
        const long long p0 = tile * kTP;
        // ---- 1. normals into Zs[k][p]: R threads per path, each drawing two
        // quads (q, q + R) at a time with their Philox rounds interleaved
        // (8 or 16 warps per SM leave little other independent work)
        {
            const int p = tid & (kTP - 1), r = tid >> 6;
            const unsigned long long path = a.path0 + (unsigned long long)(p0 + p);
            const uint32_t plo = (uint32_t)path, phi = (uint32_t)(path >> 32);
            const int days = t.aggregated ? 1 : a.horizon;
            for (int q = r; q < kpad / 4; q += 2 * R) {
                const int q2 = q + R;
                const bool has2 = q2 < kpad / 4;
                float4 z = make_float4(0.f, 0.f, 0.f, 0.f), y = make_float4(0.f, 0.f, 0.f, 0.f);
                for (int d = 0; d < days; d++) {
                    uint4 wa = make_uint4((uint32_t)(d * nq + q), 0u, plo, phi);
                    uint4 wb = make_uint4((uint32_t)(d * nq + q2), 0u, plo, phi);
                    rg_philox2(wa, wb, a.keys);
                    float z0, z1, z2, z3, y0, y1, y2, y3;
                    rg_box_muller_unscaled(wa.x, wa.y, z0, z1);
                    rg_box_muller_unscaled(wa.z, wa.w, z2, z3);
                    rg_box_muller_unscaled(wb.x, wb.y, y0, y1);
                    rg_box_muller_unscaled(wb.z, wb.w, y2, y3);
                    z.x += z0;
                    z.y += z1;
                    z.z += z2;
                    z.w += z3;
                    y.x += y0;
                    y.y += y1;
                    y.z += y2;
                    y.w += y3;
                }
                z.x *= t.zscale;
                z.y *= t.zscale;
                z.z *= t.zscale;
                z.w *= t.zscale;
                y.x *= t.zscale;
                y.y *= t.zscale;
                y.z *= t.zscale;
                y.w *= t.zscale;
                if (q >= nq) z = make_float4(0.f, 0.f, 0.f, 0.f); // padding rows
                if (q2 >= nq) y = make_float4(0.f, 0.f, 0.f, 0.f);
                Zs[(4 * q + 0) * kTP + p] = z.x;
                Zs[(4 * q + 1) * kTP + p] = z.y;
                Zs[(4 * q + 2) * kTP + p] = z.z;
                Zs[(4 * q + 3) * kTP + p] = z.w;
                if (has2) {
                    Zs[(4 * q2 + 0) * kTP + p] = y.x;
                    Zs[(4 * q2 + 1) * kTP + p] = y.y;
                    Zs[(4 * q2 + 2) * kTP + p] = y.z;
                    Zs[(4 * q2 + 3) * kTP + p] = y.w;
                }
            }
        }
        if (tid < kTP) {
            totS[tid] = 0;
            totP[tid] = 0.f;
        }
        __syncthreads();

        // ---- 2./3. column blocks
        for (int cb = 0; cb < ncb; cb++) {
            const int c0 = cb * TN;
            const int kmax = min(kpad, c0 + TN);
            // warp w holds assets c0 + 16w .. c0 + 16w + 15 (ag = 2w, 2w + 1):
            // L[c][k] = 0 for k > c, so its multiply-adds stop at c0 + 16(w + 1)
            // (the skipped terms are exact zeros; the block's staging and
            // barriers still run for every warp)
            const int kend_w = min(kmax, c0 + 16 * ((tid >> 5) + 1));
            const bool live_w = c0 + 16 * (tid >> 5) < n;
            float2 acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; i++)
#pragma unroll
                for (int j = 0; j < 4; j++) acc[i][j] = make_float2(0.f, 0.f);
            // stage slice 0 (8 rows x TN / 4 float4 per pass)
            {
                const int kk = tid / (TN / 4), c4 = tid % (TN / 4);
#pragma unroll
                for (int h = 0; h < KT; h += 8)
                    cp_async16(&Ls[(kk + h) * TN + 4 * c4], &t.Lt[(size_t)(kk + h) * t.npad + c0 + 4 * c4]);
                cp_async_commit();
            }
            int buf = 0;
            for (int k0 = 0; k0 < kmax; k0 += KT) {
                cp_async_wait_all();
                __syncthreads();
                if (k0 + KT < kmax) {
                    const int kk = tid / (TN / 4), c4 = tid % (TN / 4);
#pragma unroll
                    for (int h = 0; h < KT; h += 8)
                        cp_async16(&Ls[(buf ^ 1) * KT * TN + (kk + h) * TN + 4 * c4],
                                   &t.Lt[(size_t)(k0 + KT + kk + h) * t.npad + c0 + 4 * c4]);
                    cp_async_commit();
                }
                const float *Lb = Ls + buf * KT * TN;
                if (live_w && k0 < kend_w) {
#pragma unroll
                    for (int kk = 0; kk < KT; kk++) {
                        const float4 z = *reinterpret_cast<const float4 *>(&Zs[(k0 + kk) * kTP + 4 * pg]);
                        const float4 l0 = *reinterpret_cast<const float4 *>(&Lb[kk * TN + 8 * ag]);
                        const float4 l1 = *reinterpret_cast<const float4 *>(&Lb[kk * TN + 8 * ag + 4]);
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
                for (int g = 0; g < NAG; g++) {
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

// ---------------------------------------------------------------------------
// Warp-specialised form (RG_PLAIN_KERNEL=ws): normal generation and the GEMM run
// at the same time on different warps of one CTA per SM (512 threads).
//   warps 8-15  generator: draw the normals of a 32-path tile (Philox4x32-10
//               + Box-Muller, summed over the H days, or one N(0, H) draw per
//               asset) into one slot of a two-slot ring Zs[slot][k][p];
//   warps 0-7   GEMM: R = H mu + L Z over 256-asset column blocks, 4-path x
//               8-asset register tiles accumulated with packed __ffma2_rn,
//               L^T slices (8 x 256) staged by cp.async, double buffered.
//               Warp w holds assets c0 + 32w .. c0 + 32w + 31 of a block, so
//               its K loop stops at c0 + 32(w + 1) (L is lower triangular:
//               about 8 % of the multiply-adds at N = 600 are padding, 36 %
//               with a cut per 128-asset block), and a warp whose assets are
//               all >= N skips the block.
// Handoff by named barriers: FULL[s] (ids 2, 3) completes when the 256
// generator threads have arrived after writing slot s and the 256 GEMM
// threads sync on it; EMPTY[s] (ids 4, 5) completes when the GEMM threads
// have arrived after their last read of slot s and the generator threads
// sync on it before refilling it.  Both roles walk the same static tile
// list, so the arrivals and waits pair up by construction (the GEMM side
// skips the EMPTY arrival of its last two tiles, which nobody waits for).
// Per column block the crash counts and w.R partial sums of a warp's 32
// assets are reduced across its lanes by shuffles, then over the 8 warps in
// warp order by the path's own thread (deterministic).  Each asset's return
// is the same FMA chain in k order as in the phase-serial kernel, so S per
// path is identical between the two.
// Shared memory: 2 x 128 x Kpad bytes for Z (154 KB at N = 600) + 16 KB of
// L staging + 2 KB of partials (+ 16 KB of VaR histogram): N <= 768.
static constexpr int kWsP = 32;
static constexpr int kWsTN = 256;
static constexpr int kWsThreadsT = 512;
static constexpr int kWsHalf = 256;

__device__ __forceinline__ void nbar_sync(int id, int count)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}
__device__ __forceinline__ void nbar_arrive(int id, int count)
{
    asm volatile("bar.arrive %0, %1;" ::"r"(id), "r"(count) : "memory");
}

template <bool VAR>
__global__ void __launch_bounds__(kWsThreadsT, 1) mc_tiled_ws_kernel(const TiledArgs t)
{
    extern __shared__ __align__(16) float smem[];
    const PlainArgs &a = t.a;
    const int kpad = t.kpad;
    float *Zs = smem;                                  // [2][kpad][kWsP]
    float *Ls = Zs + 2 * (size_t)kpad * kWsP;          // [2][kTK][kWsTN]
    int *partS = (int *)(Ls + 2 * kTK * kWsTN);        // [8][kWsP]
    float *partP = (float *)(partS + 8 * kWsP);        // [8][kWsP]
    __shared__ unsigned long long sacc[4];
    __shared__ unsigned int shist[VAR ? kVarHistBins + 2 : 1];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    if (tid < 4) sacc[tid] = 0ull;
    if (VAR && a.var_mode == 2)
        for (int i = tid; i < a.sel_bins + 2; i += blockDim.x) shist[i] = 0u;
    __syncthreads();
    int crash = 0, breach = 0, n_tail = 0;
    long long tail_fx = 0;
    const int n = a.n;
    const int nq = (n + 3) >> 2;
    const long long ntiles = (a.n_paths + kWsP - 1) / kWsP;
    const long long my_tiles = (long long)blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (warp >= 8) {
        // ============================ generator ============================
        const int gt = tid - kWsHalf;
        const int days = t.aggregated ? 1 : a.horizon;
        const int items = kWsP * (kpad / 4);
        for (long long j = 0; j < my_tiles; j++) {
            const int s = (int)(j & 1);
            if (j >= 2) nbar_sync(4 + s, kWsThreadsT); // slot s released by the GEMM warps
            const long long p0 = ((long long)blockIdx.x + j * gridDim.x) * kWsP;
            float *Z = Zs + (size_t)s * kpad * kWsP;
            for (int it = gt; it < items; it += kWsHalf) {
                const int p = it & (kWsP - 1), q = it >> 5;
                float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
                if (q < nq) {
                    const unsigned long long path = a.path0 + (unsigned long long)(p0 + p);
                    const uint32_t plo = (uint32_t)path, phi = (uint32_t)(path >> 32);
                    for (int d = 0; d < days; d++) {
                        const uint4 wv = rg_philox(make_uint4((uint32_t)(d * nq + q), 0u, plo, phi), a.keys);
                        float z0, z1, z2, z3;
                        rg_box_muller_unscaled(wv.x, wv.y, z0, z1);
                        rg_box_muller_unscaled(wv.z, wv.w, z2, z3);
                        z.x += z0;
                        z.y += z1;
                        z.z += z2;
                        z.w += z3;
                    }
                    z.x *= t.zscale;
                    z.y *= t.zscale;
                    z.z *= t.zscale;
                    z.w *= t.zscale;
                }
                Z[(4 * q + 0) * kWsP + p] = z.x;
                Z[(4 * q + 1) * kWsP + p] = z.y;
                Z[(4 * q + 2) * kWsP + p] = z.z;
                Z[(4 * q + 3) * kWsP + p] = z.w;
            }
            __threadfence_block();
            nbar_arrive(2 + s, kWsThreadsT); // slot s full
        }
    } else {
        // ============================== GEMM ===============================
        const int pg = tid & 7, ag = tid >> 3; // paths 4pg..4pg+3; assets 8ag..8ag+7 of a block
        const int ncb = (n + kWsTN - 1) / kWsTN;
        for (long long j = 0; j < my_tiles; j++) {
            const int s = (int)(j & 1);
            nbar_sync(2 + s, kWsThreadsT); // slot s full
            const long long p0 = ((long long)blockIdx.x + j * gridDim.x) * kWsP;
            const float *Z = Zs + (size_t)s * kpad * kWsP;
            int totS = 0;      // threads 0..31: path p0 + tid
            float totP = 0.f;
            for (int cb = 0; cb < ncb; cb++) {
                const int c0 = cb * kWsTN;
                const int kmax = min(kpad, c0 + kWsTN);
                const int wlo = c0 + 32 * warp;
                const int kend = min(kpad, wlo + 32);
                const bool active = wlo < n;
                float2 acc[4][4];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) acc[i][jj] = make_float2(0.f, 0.f);
                const int sk = tid >> 5, sc = tid & 31; // staging: row sk, columns 8sc..8sc+7
                cp_async16(&Ls[sk * kWsTN + 8 * sc], &t.Lt[(size_t)sk * t.npad + c0 + 8 * sc]);
                cp_async16(&Ls[sk * kWsTN + 8 * sc + 4], &t.Lt[(size_t)sk * t.npad + c0 + 8 * sc + 4]);
                cp_async_commit();
                int buf = 0;
                for (int k0 = 0; k0 < kmax; k0 += kTK) {
                    cp_async_wait_all();
                    nbar_sync(1, kWsHalf);
                    if (k0 + kTK < kmax) {
                        float *dst = Ls + (buf ^ 1) * kTK * kWsTN + sk * kWsTN + 8 * sc;
                        const float *src = &t.Lt[(size_t)(k0 + kTK + sk) * t.npad + c0 + 8 * sc];
                        cp_async16(dst, src);
                        cp_async16(dst + 4, src + 4);
                        cp_async_commit();
                    }
                    if (active && k0 < kend) {
                        const float *Lb = Ls + buf * kTK * kWsTN;
#pragma unroll
                        for (int kk = 0; kk < kTK; kk++) {
                            const float4 z = *reinterpret_cast<const float4 *>(&Z[(k0 + kk) * kWsP + 4 * pg]);
                            const float4 l0 = *reinterpret_cast<const float4 *>(&Lb[kk * kWsTN + 8 * ag]);
                            const float4 l1 = *reinterpret_cast<const float4 *>(&Lb[kk * kWsTN + 8 * ag + 4]);
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
                    }
                    buf ^= 1;
                }
                // block epilogue: this thread's 4 paths x 8 assets, then the
                // warp's 4 asset groups (lanes pg, pg+8, pg+16, pg+24)
                float hm[8], wt[8];
#pragma unroll
                for (int jj = 0; jj < 8; jj++) {
                    const int c = c0 + 8 * ag + jj;
                    hm[jj] = (c < n) ? (float)((double)a.horizon * a.mu64[c]) : 0.f;
                    wt[jj] = (c < n) ? a.w[c] : 0.f;
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    int sv = 0;
                    float pw = 0.f;
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) {
                        const int a0 = c0 + 8 * ag + 2 * jj;
                        const float r0 = hm[2 * jj] + acc[i][jj].x;
                        const float r1 = hm[2 * jj + 1] + acc[i][jj].y;
                        sv += (a0 < n && r0 < a.neg_x) ? 1 : 0;
                        sv += (a0 + 1 < n && r1 < a.neg_x) ? 1 : 0;
                        pw = fmaf(wt[2 * jj], r0, pw);
                        pw = fmaf(wt[2 * jj + 1], r1, pw);
                    }
                    sv += __shfl_xor_sync(0xffffffffu, sv, 8);
                    pw += __shfl_xor_sync(0xffffffffu, pw, 8);
                    sv += __shfl_xor_sync(0xffffffffu, sv, 16);
                    pw += __shfl_xor_sync(0xffffffffu, pw, 16);
                    if (lane < 8) {
                        partS[warp * kWsP + 4 * pg + i] = sv;
                        partP[warp * kWsP + 4 * pg + i] = pw;
                    }
                }
                nbar_sync(1, kWsHalf);
                if (tid < kWsP) {
#pragma unroll
                    for (int w = 0; w < 8; w++) {
                        totS += partS[w * kWsP + tid];
                        totP += partP[w * kWsP + tid];
                    }
                }
                // partS / partP are rewritten only after the next block's
                // first barrier; Ls only after this one
            }
            // every read of slot s is done: the generator may refill it
            if (j + 2 < my_tiles) nbar_arrive(4 + s, kWsThreadsT);
            if (tid < kWsP) {
                const long long p = p0 + tid;
                if (p < a.n_paths) {
                    crash += (totS >= a.k) ? 1 : 0;
                    breach += (a.has_w && totP < a.port_thr) ? 1 : 0;
                    if (a.s_values) a.s_values[p] = totS;
                    if (a.port_values) a.port_values[p] = totP;
                    if (VAR) var_path(a, totP, shist, n_tail, tail_fx);
                }
            }
        }
    }
    cta_flush(a, crash, breach, n_tail, tail_fx, sacc, VAR ? shist : nullptr, VAR);
}

// ---------------------------------------------------------------------------
// Pipelined form (the default): the phase-serial kernel's tile (64
// paths, one Z buffer) with generation and GEMM on different warps of one
// 512-thread CTA, overlapped through the 128-row ranges of Z.
//   warps 0-7  GEMM: column blocks in DESCENDING order and, inside a block,
//              K in DESCENDING order.  Block cb reads rows [0, 128(cb + 1)),
//              its own range [128 cb, 128(cb + 1)) first; blocks below cb
//              never read that range, so it is released (RELEASE[cb]) as soon
//              as the block's K loop has passed it.  The next tile's first
//              block (the top one) reads the ranges top down, the order in
//              which they were released, waiting on FILLED[r] as it enters
//              range r.
//   warps 8-15 normals of the next tile, range by range from the top
//              (waiting on RELEASE[r], then arriving on FILLED[r]); two quads
//              at a time with their Philox rounds interleaved (rg_philox2).
// At N = 600 the bottom range, released last, is needed only at the end of
// the next tile's top block, so generation and GEMM overlap almost entirely.
// The GEMM is the phase-serial kernel's (4-path x 8-asset FFMA2 tiles,
// L^T slices of KT = 32 rows where shared memory allows, else 16 or 8,
// staged by cp.async, per-warp triangle cut) with a barrier among the GEMM
// warps only.  Each return is the same terms as in
// the other forms, accumulated in descending k.
// Named barriers, pairing by construction (both roles walk the same static
// tile list and block count): 1 = GEMM warps (256); 2 + r = FILLED[r] (256
// generator arrivals + 256 GEMM syncs, once a tile); 8 + r = RELEASE[r] (256
// GEMM arrivals in every tile but the CTA's last + 256 generator syncs in
// every tile but the first); r < 6 (N <= 768).
static constexpr int kPipeThreads = 512;
static constexpr int kPipeHalf = 256;

template <bool VAR, int KT>
__global__ void __launch_bounds__(kPipeThreads, 1) mc_tiled_pipe_kernel(const TiledArgs t)
{
    extern __shared__ __align__(16) float smem[];
    const PlainArgs &a = t.a;
    const int kpad = t.kpad;
    float *Zs = smem;                                  // [kpad][kTP]
    float *Ls = Zs + (size_t)kpad * kTP;               // [2][KT][kTN]
    int *partS = (int *)(Ls + 2 * KT * kTN);           // [16][kTP]
    float *partP = (float *)(partS + 16 * kTP);        // [16][kTP]
    __shared__ unsigned long long sacc[4];
    __shared__ unsigned int shist[VAR ? kVarHistBins + 2 : 1];
    __shared__ float s_hmu[kTiledMaxN];                // H mu_c rounded to FP32, once per CTA

    const int tid = threadIdx.x;
    if (tid < 4) sacc[tid] = 0ull;
    if (VAR && a.var_mode == 2)
        for (int i = tid; i < a.sel_bins + 2; i += blockDim.x) shist[i] = 0u;
    for (int c = tid; c < a.n; c += blockDim.x) s_hmu[c] = (float)((double)a.horizon * a.mu64[c]);
    __syncthreads();
    int crash = 0, breach = 0, n_tail = 0;
    long long tail_fx = 0;
    const int n = a.n;
    const int nq = (n + 3) >> 2;
    const int ncb = (n + kTN - 1) / kTN;
    const long long ntiles = (a.n_paths + kTP - 1) / kTP;
    const long long my_tiles = (long long)blockIdx.x < ntiles ? (ntiles - 1 - blockIdx.x) / gridDim.x + 1 : 0;

    if (tid >= kPipeHalf) {
        // ============================ generator ============================
        const int gt = tid - kPipeHalf;
        const int p = gt & (kTP - 1), r4 = gt >> 6; // 4 threads per path
        const int days = t.aggregated ? 1 : a.horizon;
        for (long long j = 0; j < my_tiles; j++) {
            const long long p0 = ((long long)blockIdx.x + j * gridDim.x) * kTP;
            const unsigned long long path = a.path0 + (unsigned long long)(p0 + p);
            const uint32_t plo = (uint32_t)path, phi = (uint32_t)(path >> 32);
            for (int r = ncb - 1; r >= 0; r--) {
                if (j >= 1) nbar_sync(8 + r, kPipeThreads); // range r of the previous tile is dead
                const int qlo = 32 * r, qhi = min(kpad / 4, 32 * r + 32);
                for (int q = qlo + r4; q < qhi; q += 8) {
                    const int q2 = q + 4;
                    const bool has2 = q2 < qhi;
                    float4 z = make_float4(0.f, 0.f, 0.f, 0.f), y = make_float4(0.f, 0.f, 0.f, 0.f);
                    for (int d = 0; d < days; d++) {
                        uint4 wa = make_uint4((uint32_t)(d * nq + q), 0u, plo, phi);
                        uint4 wb = make_uint4((uint32_t)(d * nq + q2), 0u, plo, phi);
                        rg_philox2(wa, wb, a.keys);
                        float z0, z1, z2, z3, y0, y1, y2, y3;
                        rg_box_muller_unscaled(wa.x, wa.y, z0, z1);
                        rg_box_muller_unscaled(wa.z, wa.w, z2, z3);
                        rg_box_muller_unscaled(wb.x, wb.y, y0, y1);
                        rg_box_muller_unscaled(wb.z, wb.w, y2, y3);
                        z.x += z0;
                        z.y += z1;
                        z.z += z2;
                        z.w += z3;
                        y.x += y0;
                        y.y += y1;
                        y.z += y2;
                        y.w += y3;
                    }
                    z.x *= t.zscale;
                    z.y *= t.zscale;
                    z.z *= t.zscale;
                    z.w *= t.zscale;
                    y.x *= t.zscale;
                    y.y *= t.zscale;
                    y.z *= t.zscale;
                    y.w *= t.zscale;
                    if (q >= nq) z = make_float4(0.f, 0.f, 0.f, 0.f); // padding rows
                    if (q2 >= nq) y = make_float4(0.f, 0.f, 0.f, 0.f);
                    Zs[(4 * q + 0) * kTP + p] = z.x;
                    Zs[(4 * q + 1) * kTP + p] = z.y;
                    Zs[(4 * q + 2) * kTP + p] = z.z;
                    Zs[(4 * q + 3) * kTP + p] = z.w;
                    if (has2) {
                        Zs[(4 * q2 + 0) * kTP + p] = y.x;
                        Zs[(4 * q2 + 1) * kTP + p] = y.y;
                        Zs[(4 * q2 + 2) * kTP + p] = y.z;
                        Zs[(4 * q2 + 3) * kTP + p] = y.w;
                    }
                }
                __threadfence_block();
                nbar_arrive(2 + r, kPipeThreads); // range r of this tile written
            }
        }
    } else {
        // ============================== GEMM ===============================
        const int pg = tid & 15, ag = tid >> 4;
        const int kk0 = tid >> 5, c4 = tid & 31; // staging: 8 rows x 32 float4 per pass
        for (long long j = 0; j < my_tiles; j++) {
            const long long p0 = ((long long)blockIdx.x + j * gridDim.x) * kTP;
            const bool has_next = j + 1 < my_tiles;
            int totS = 0;   // threads 0..63: path p0 + tid
            float totP = 0.f;
            for (int cb = ncb - 1; cb >= 0; cb--) {
                const int c0 = cb * kTN;
                const int kmax = min(kpad, c0 + kTN);
                const int kend_w = min(kmax, c0 + 16 * ((tid >> 5) + 1));
                const bool live_w = c0 + 16 * (tid >> 5) < n;
                float2 acc[4][4];
#pragma unroll
                for (int i = 0; i < 4; i++)
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) acc[i][jj] = make_float2(0.f, 0.f);
                // K descending: slices kmax - KT, kmax - 2 KT, ..., 0
                const int ktop = kmax - KT;
#pragma unroll
                for (int h = 0; h < KT; h += 8)
                    cp_async16(&Ls[(kk0 + h) * kTN + 4 * c4], &t.Lt[(size_t)(ktop + kk0 + h) * t.npad + c0 + 4 * c4]);
                cp_async_commit();
                int buf = 0;
                for (int k0 = ktop; k0 >= 0; k0 -= KT) {
                    cp_async_wait_all();
                    nbar_sync(1, kPipeHalf);
                    // every GEMM warp is past slice k0 + KT: entering a new
                    // range (k0 + KT a multiple of 128) releases the one above
                    // it if that is this block's own range
                    if (has_next && k0 + KT == c0) nbar_arrive(8 + cb, kPipeThreads);
                    // the top block reads every range first in this tile
                    if (cb == ncb - 1 && (k0 + KT) % kTN == 0 || (cb == ncb - 1 && k0 == ktop))
                        nbar_sync(2 + k0 / kTN, kPipeThreads);
                    if (k0 - KT >= 0) {
#pragma unroll
                        for (int h = 0; h < KT; h += 8)
                            cp_async16(&Ls[(buf ^ 1) * KT * kTN + (kk0 + h) * kTN + 4 * c4],
                                       &t.Lt[(size_t)(k0 - KT + kk0 + h) * t.npad + c0 + 4 * c4]);
                        cp_async_commit();
                    }
                    const float *Lb = Ls + buf * KT * kTN;
                    if (live_w && k0 < kend_w) {
#pragma unroll
                        for (int kk = KT - 1; kk >= 0; kk--) {
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
                    }
                    buf ^= 1;
                }
                float hm[8], wt[8];
#pragma unroll
                for (int jj = 0; jj < 8; jj++) {
                    const int c = c0 + 8 * ag + jj;
                    hm[jj] = (c < n) ? s_hmu[c] : 0.f;
                    wt[jj] = (c < n) ? a.w[c] : 0.f;
                }
#pragma unroll
                for (int i = 0; i < 4; i++) {
                    int sv = 0;
                    float pw = 0.f;
#pragma unroll
                    for (int jj = 0; jj < 4; jj++) {
                        const int a0 = c0 + 8 * ag + 2 * jj;
                        const float r0 = hm[2 * jj] + acc[i][jj].x;
                        const float r1 = hm[2 * jj + 1] + acc[i][jj].y;
                        sv += (a0 < n && r0 < a.neg_x) ? 1 : 0;
                        sv += (a0 + 1 < n && r1 < a.neg_x) ? 1 : 0;
                        pw = fmaf(wt[2 * jj], r0, pw);
                        pw = fmaf(wt[2 * jj + 1], r1, pw);
                    }
                    partS[ag * kTP + 4 * pg + i] = sv;
                    partP[ag * kTP + 4 * pg + i] = pw;
                }
                nbar_sync(1, kPipeHalf); // every GEMM warp is past block cb: Ls and the partials are free
                if (has_next && c0 == 0) nbar_arrive(8 + cb, kPipeThreads); // block 0's range, passed last
                if (tid < kTP) {
#pragma unroll
                    for (int g = 0; g < 16; g++) {
                        totS += partS[g * kTP + tid];
                        totP += partP[g * kTP + tid];
                    }
                }
                // partS / partP are rewritten only after the next block's
                // first barrier
            }
            if (tid < kTP) {
                const long long p = p0 + tid;
                if (p < a.n_paths) {
                    crash += (totS >= a.k) ? 1 : 0;
                    breach += (a.has_w && totP < a.port_thr) ? 1 : 0;
                    if (a.s_values) a.s_values[p] = totS;
                    if (a.port_values) a.port_values[p] = totP;
                    if (VAR) var_path(a, totP, shist, n_tail, tail_fx);
                }
            }
        }
    }
    cta_flush(a, crash, breach, n_tail, tail_fx, sacc, VAR ? shist : nullptr, VAR);
}

int tiled_max_n() { return kTiledMaxN; }

size_t tiled_smem_bytes(int n, int kt, int threads)
{
    const int kpad = tiled_kpad(n);
    return sizeof(float) * ((size_t)kpad * kTP + 2 * (size_t)kt * (threads / 2) + 2 * (size_t)(threads / 16) * kTP);
}

size_t tiled_ws_smem_bytes(int n)
{
    const int kpad = tiled_kpad(n);
    return sizeof(float) * (2 * (size_t)kpad * kWsP + 2 * kTK * kWsTN + 2 * 8 * kWsP);
}

// npad is a multiple of both column-block widths (128 and 256)
int tiled_npad(int n) { return (n + kWsTN - 1) / kWsTN * kWsTN; }
// K padded to 32: an L^T slice (up to 32 rows) never reads past the last
// row, and a descending K loop ends exactly at row 0
int tiled_kpad(int n) { return (n + 31) / 32 * 32; }

// The pipelined kernel unless RG_PLAIN_KERNEL names "serial" (the
// phase-serial kernel) or "ws" (the warp-specialised kernel), both kept for
// comparison.
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
    t.zscale = (float)((double)kBmScale * (aggregated ? std::sqrt((double)a.horizon) : 1.0));
    const char *env = getenv("RG_PLAIN_KERNEL");
    const bool ws = env && strstr(env, "ws") != nullptr;
    const bool serial = env && strstr(env, "serial") != nullptr;
    if (!ws && !serial) {
        int dev = 0, optin = 0;
        cudaError_t e = cudaGetDevice(&dev);
        if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
        if (e != cudaSuccess) return e;
        const bool var = a.var_mode != 0;
        const size_t static_bytes =
            1024 + 4 * (size_t)kTiledMaxN + (var ? 4 * (size_t)(kVarHistBins + 2) : 0); // + s_hmu
        // the widest L^T slice (32, 16 or 8 rows) whose shared memory fits
        const int kt = tiled_smem_bytes(a.n, 32, kTiledThreads) + static_bytes <= (size_t)optin   ? 32
                       : tiled_smem_bytes(a.n, 16, kTiledThreads) + static_bytes <= (size_t)optin ? 16
                                                                                                  : 8;
        const size_t smem = tiled_smem_bytes(a.n, kt, kTiledThreads);
        void (*kern)(const TiledArgs) =
            var ? (kt == 32 ? mc_tiled_pipe_kernel<true, 32>
                            : kt == 16 ? mc_tiled_pipe_kernel<true, 16> : mc_tiled_pipe_kernel<true, 8>)
                : (kt == 32 ? mc_tiled_pipe_kernel<false, 32>
                            : kt == 16 ? mc_tiled_pipe_kernel<false, 16> : mc_tiled_pipe_kernel<false, 8>);
        e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        long long tiles = (a.n_paths + kTP - 1) / kTP;
        long long grid = sm_count;
        if (tiles < grid) grid = tiles;
        kern<<<(unsigned)grid, kPipeThreads, smem, s>>>(t);
        return cudaGetLastError();
    }
    if (ws) {
        const size_t smem = tiled_ws_smem_bytes(a.n);
        auto kern = (a.var_mode != 0) ? mc_tiled_ws_kernel<true> : mc_tiled_ws_kernel<false>;
        cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        long long tiles = (a.n_paths + kWsP - 1) / kWsP;
        long long grid = sm_count;
        if (tiles < grid) grid = tiles;
        kern<<<(unsigned)grid, kWsThreadsT, smem, s>>>(t);
        return cudaGetLastError();
    }
    // 16-row L^T slices where the CTA's shared memory (dynamic + static)
    // fits, else 8
    int dev = 0, optin = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev);
    if (e != cudaSuccess) return e;
    const bool var = a.var_mode != 0;
    const size_t static_bytes = 1024 + (var ? 4 * (size_t)(kVarHistBins + 2) : 0);
    const int threads = kTiledThreads;
    const bool kt16 = tiled_smem_bytes(a.n, 16, threads) + static_bytes <= (size_t)optin;
    const size_t smem = tiled_smem_bytes(a.n, kt16 ? 16 : 8, threads);
    void (*kern)(const TiledArgs) =
        var ? (kt16 ? mc_tiled_kernel<true, 16, kTiledThreads> : mc_tiled_kernel<true, 8, kTiledThreads>)
            : (kt16 ? mc_tiled_kernel<false, 16, kTiledThreads> : mc_tiled_kernel<false, 8, kTiledThreads>);
    e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    long long tiles = (a.n_paths + kTP - 1) / kTP;
    long long grid = sm_count;
    if (tiles < grid) grid = tiles;
    kern<<<(unsigned)grid, threads, smem, s>>>(t);
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
