// Precision form: the correlation step on tcgen05 tensor cores.
//
// Computes what the plain kernels compute (R = H mu + L Zsum per path, S,
// w.R, crash / breach / VaR bookkeeping) with the contraction as a dense
// MMA on sm_103a tensor cores, in transposed form so that a path tile's
// normals fit on chip:
//
//     D[asset, path] = sum_k Lhat[asset, k] * Z[path, k]      (tcgen05.mma)
//
// M = 128 asset rows per MMA (n_mt = ceil((N+1)/128) row tiles), N = P paths
// per tile, K = 16 per instruction, FP32 accumulators in tensor memory
// (n_mt x P columns, <= 512).  Row N of Lhat is w^T L, so the portfolio
// return w.R = H w.mu + D[N, path] comes out of the same MMAs.
//
// Precision: both operands are split into FP16 (or BF16) hi + lo parts and
// three products are accumulated, Lhi.Zhi + Lhi.Zlo + Llo.Zhi (the lo.lo term
// is below FP32 rounding for FP16).  L is scaled by 2^8 so its lo part stays
// in FP16's normal range; the epilogue scales back exactly.
//
// Two kernels, one CTA per SM, persistent over path tiles:
//   mc_tcws_kernel   (the engine's default) warp-specialised, 1024 threads:
//                    26 generator warps draw the next tile's normals into a
//                    ring of K-tile slots while one thread streams the
//                    pre-swizzled Lhat tiles (cp.async.bulk, mbarrier ring),
//                    one thread issues the MMAs K-tile-outer, and four warps
//                    read each row tile's accumulators (tcgen05.ld) as soon
//                    as it is complete.  P = 128 paths up to N = 511, 96
//                    up to N = 639, else 64 (tensor-memory columns).
//   mc_tc_kernel     phase-serial, 512 threads, P = 64: all threads draw the
//                    tile's normals, one thread streams Lhat through a
//                    2-stage ring while another issues the MMAs row tile by
//                    row tile, then all 16 warps read the accumulators.
// Every wait is bounded: on expiry the kernel sets an error word, drains its
// own copies and MMAs (again bounded), frees its tensor memory and returns;
// the host reports RG_ERR_TIMEOUT.
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <cuda_fp16.h>
#include <cuda_bf16.h>
#include "rg_fused_kernel.cuh"

namespace rg {

static constexpr int kTcPaths = 64;        // N of the MMA: paths per tile
static constexpr int kTcRows = 128;        // M of the MMA: asset rows per row tile
static constexpr int kTcKt = 64;           // K elements per shared-memory tile (128 B)
static constexpr int kTcThreads = 512;
static constexpr int kTcMaxKt = 10;        // K tiles of Z kept on chip (N <= 640)
static constexpr int kTcStages = 2;
static constexpr int kTcTileBytes = kTcRows * kTcKt * 2;  // one part of an Lhat tile: 16 KB
static constexpr int kTcZBytes = kTcPaths * kTcKt * 2;    // one part of a Z K tile: 8 KB
static constexpr float kTcLScale = 256.0f;
static constexpr unsigned kTcSpinLimit = 1u << 26;        // try_wait polls before giving up
static constexpr unsigned long long kTcWaitNs = 2000000000ull; // 2 s of wall time
static constexpr unsigned kTcSuspendNs = 1u << 16;           // try_wait suspend hint (65 us)

// One (portfolio, query) of a launch.  Tiles of 64 paths are numbered
// globally across the items of a launch; item i owns tiles
// [tile_begin, tile_begin + ceil(n_paths / 64)).
struct TcItem {
    const unsigned char *tiles;   // pre-swizzled Lhat of the portfolio
    const double *mu64;           // daily means
    unsigned long long *counts;   // [2] crash, breach of this item
    int *s_values;                // optional per-path outputs (item-local)
    float *port_values;
    unsigned long long path0;     // first path index of the query
    long long n_paths;
    long long tile_begin;
    PhiloxKeys keys;
    double hwmu;                  // H w.mu
    int n, n_mt, n_kt, horizon, k, has_w, aggregated, bf16;
    float neg_x, port_thr, hwmu_f;  // hwmu_f = (float) hwmu
    float zscale;  // factor of each summed normal: sqrt(2 ln 2) (the draws are unscaled), x sqrt(H) aggregated
};

struct TcBatch {
    const TcItem *items;      // device array (batches), or null: use `one`
    TcItem one;               // single item passed by value
    int n_items;
    int unit_tiles;           // tiles per work unit
    long long total_tiles;
    unsigned int *work;       // unit counter (dynamic scheduling), or null: static
    unsigned int *err;        // device error word
    int inject_stall;         // host-side fault injection: one stage is never filled
    int n_kt_max;             // K tiles of the largest item (shared-memory size)
    int tmem_cols;            // tensor-memory columns allocated (power of 2 >= 64 n_mt_max)
    const long long *dyn;     // if set: [0] items, [1] total tiles, read from device memory
                              // (a graph captured once serves batches of any size)
    PlainArgs var;            // VaR fields of a single-item query (var_mode 0 otherwise)
};

// Scaled crash threshold of asset row r: the accumulator D = 2^8 (L Z)_r is
// compared with 2^8 (-x - H mu_r).  FP32 throughout, like the epilogue's
// portfolio value: this part's FP64 pipe is narrow, and one FP32 rounding
// of these terms is far below the tensor-core form's own error.
__device__ __forceinline__ float tc_threshold(const TcItem &it, int r)
{
    return (it.neg_x - (float)it.horizon * (float)it.mu64[r]) * kTcLScale;
}

// ------------------------------------------------------------ PTX wrappers
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, unsigned parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
// The same with a suspend-time hint: a waiting thread sleeps until the phase
// completes or about `ns` nanoseconds pass, instead of the hardware's
// shorter default, so long waits cost few polls (issue slots).
__device__ __forceinline__ bool mbar_try_wait_hint(uint64_t *bar, unsigned parity, unsigned ns)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity), "r"(ns)
                 : "memory");
    return ok != 0;
}
// Non-blocking probe of a phase (mbarrier.test_wait never suspends).
__device__ __forceinline__ bool mbar_test(uint64_t *bar, unsigned parity)
{
    uint32_t ok;
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
                 "selp.u32 %0, 1, 0, p;\n\t}"
                 : "=r"(ok)
                 : "r"(smem_u32(bar)), "r"(parity)
                 : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
// Bounded wait: gives up (returns false) after kTcWaitNs of wall time or
// kTcSpinLimit polls, whichever comes first.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity)
{
    if (mbar_try_wait(bar, parity)) return true; // common case: no timer read
    const unsigned long long t0 = global_ns();
    for (unsigned i = 0; i < kTcSpinLimit; i++) {
        if (mbar_try_wait_hint(bar, parity, kTcSuspendNs)) return true;
        if ((i & 15u) == 15u && global_ns() - t0 > kTcWaitNs) return false;
    }
    return false;
}
__device__ __forceinline__ void bulk_copy(void *smem_dst, const void *gmem_src, unsigned bytes, uint64_t *bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(smem_dst)),
                 "l"(gmem_src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void fence_async_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major, 128-byte swizzle, 8-row groups
// 1024 bytes apart.
__host__ __device__ constexpr uint64_t sw128_desc(uint32_t addr)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);  // start address
    d |= (uint64_t)1 << 16;                   // leading byte offset (unused by this layout)
    d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                   // descriptor version
    d |= (uint64_t)2 << 61;                   // 128-byte swizzle
    return d;
}

// The same descriptor as two words: the high word is constant and the low
// word is (address >> 4) | leading-byte-offset field, so an address step of
// 16 n bytes is + n on the low word (shared addresses stay below 2^18).
static constexpr uint32_t kSw128DescHi = (uint32_t)(sw128_desc(0u) >> 32);
__host__ __device__ constexpr uint32_t sw128_desc_lo(uint32_t addr) { return (uint32_t)sw128_desc(addr); }
static_assert(((uint64_t)kSw128DescHi << 32 | sw128_desc_lo(0x12340u)) == sw128_desc(0x12340u), "descriptor split");
static_assert(sw128_desc_lo(0x12340u + 32u) == sw128_desc_lo(0x12340u) + 2u, "K step on the low word");

// Instruction descriptor of kind::f16: FP32 accumulator, A and B of the same
// type (FP16 or BF16), both K-major, M x N.
__host__ __device__ constexpr uint32_t tc_idesc(int bf16, int M, int N)
{
    return (1u << 4) | ((uint32_t)bf16 << 7) | ((uint32_t)bf16 << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc, uint32_t idesc,
                                       uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\t"
                 "setp.ne.b32 p, %4, 0;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
                 "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate));
}
// The 12 MMAs of one (row tile, K tile) pair in one block: for each of the
// four 16-element K steps, Lhi.Zhi (accumulating unless acc_first == 0 on the
// first step), Lhi.Zlo and Llo.Zhi.  Descriptors are passed as their low
// words (sw128_desc_lo); a K step is 32 bytes (+2), the lo part of an Lhat
// tile 16 KB (+1024) further.
__device__ __forceinline__ void tc_mma_pair(uint32_t d_tmem, uint32_t a_lo, uint32_t zh_lo, uint32_t zl_lo,
                                            uint32_t idesc, uint32_t acc_first)
{
    asm volatile("{\n\t.reg .pred p, q;\n\t.reg .b32 ta, tl, th, tz;\n\t.reg .b64 da, dl, dh, dz;\n\t"
                 "setp.ne.b32 p, %5, 0;\n\t"
                 "setp.eq.b32 q, %5, %5;\n\t"
                 "add.u32 ta, %1, 0;\n\tadd.u32 tl, %1, 1024;\n\tadd.u32 th, %2, 0;\n\tadd.u32 tz, %3, 0;\n\t"
                 "mov.b64 da, {ta, %6};\n\tmov.b64 dl, {tl, %6};\n\tmov.b64 dh, {th, %6};\n\tmov.b64 dz, {tz, %6};\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, dh, %4, p;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, dz, %4, q;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], dl, dh, %4, q;\n\t"
                 "add.u32 ta, %1, 2;\n\tadd.u32 tl, %1, 1026;\n\tadd.u32 th, %2, 2;\n\tadd.u32 tz, %3, 2;\n\t"
                 "mov.b64 da, {ta, %6};\n\tmov.b64 dl, {tl, %6};\n\tmov.b64 dh, {th, %6};\n\tmov.b64 dz, {tz, %6};\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, dh, %4, q;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, dz, %4, q;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], dl, dh, %4, q;\n\t"
                 "add.u32 ta, %1, 4;\n\tadd.u32 tl, %1, 1028;\n\tadd.u32 th, %2, 4;\n\tadd.u32 tz, %3, 4;\n\t"
                 "mov.b64 da, {ta, %6};\n\tmov.b64 dl, {tl, %6};\n\tmov.b64 dh, {th, %6};\n\tmov.b64 dz, {tz, %6};\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, dh, %4, q;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, dz, %4, q;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], dl, dh, %4, q;\n\t"
                 "add.u32 ta, %1, 6;\n\tadd.u32 tl, %1, 1030;\n\tadd.u32 th, %2, 6;\n\tadd.u32 tz, %3, 6;\n\t"
                 "mov.b64 da, {ta, %6};\n\tmov.b64 dl, {tl, %6};\n\tmov.b64 dh, {th, %6};\n\tmov.b64 dz, {tz, %6};\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, dh, %4, q;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], da, dz, %4, q;\n\t"
                 "tcgen05.mma.cta_group::1.kind::f16 [%0], dl, dh, %4, q;\n\t"
                 "}"
                 ::"r"(d_tmem), "r"(a_lo), "r"(zh_lo), "r"(zl_lo), "r"(idesc), "r"(acc_first), "r"(kSw128DescHi));
}
__device__ __forceinline__ void tc_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// Byte offset of element (row r, k) in a K-major 128B-swizzled block of
// 2-byte elements, 64 elements per row.
__host__ __device__ __forceinline__ uint32_t sw128_offset(int r, int k)
{
    const int chunk = (k >> 3) ^ (r & 7);
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + chunk * 16 + (k & 7) * 2);
}

// Normals of quad q of one path summed over `days` draws (Philox counter
// (d * nq + q, 0, path lo, path hi)), divided by sqrt(2 ln 2): the caller
// scales each sum once (TcItem::zscale).  The paired form draws two quads
// (of one path or two) with their Philox rounds interleaved and gives the
// same sums.
__device__ __forceinline__ float4 tc_quad_sum(int q, int nq, int days, uint32_t plo, uint32_t phi,
                                              const PhiloxKeys &keys)
{
    float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int d = 0; d < days; d++) {
        const uint4 wv = rg_philox(make_uint4((uint32_t)(d * nq + q), 0u, plo, phi), keys);
        float z0, z1, z2, z3;
        rg_box_muller_unscaled(wv.x, wv.y, z0, z1);
        rg_box_muller_unscaled(wv.z, wv.w, z2, z3);
        z.x += z0;
        z.y += z1;
        z.z += z2;
        z.w += z3;
    }
    return z;
}
__device__ __forceinline__ void tc_quad_sum2(int q, uint32_t plo, uint32_t phi, int q2, uint32_t plo2, uint32_t phi2,
                                             int nq, int days, const PhiloxKeys &keys, float4 &z, float4 &y)
{
    z = make_float4(0.f, 0.f, 0.f, 0.f);
    y = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int d = 0; d < days; d++) {
        uint4 wa = make_uint4((uint32_t)(d * nq + q), 0u, plo, phi);
        uint4 wb = make_uint4((uint32_t)(d * nq + q2), 0u, plo2, phi2);
        rg_philox2(wa, wb, keys);
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
}

// Two FP32 values rounded to nearest and packed: a in bits 0-15, b in 16-31
// (cvt's first source goes to the upper half).
__device__ __forceinline__ uint32_t pack_bf16x2(float a, float b)
{
    uint32_t d;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
    return d;
}
__device__ __forceinline__ uint32_t pack_f16x2(float a, float b)
{
    uint32_t d;
    asm("cvt.rn.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(b), "f"(a));
    return d;
}
__device__ __forceinline__ float2 unpack_f16x2(uint32_t d)
{
    float2 r;
    asm("{\n\t.reg .b16 l, h;\n\tmov.b32 {l, h}, %2;\n\tcvt.f32.f16 %0, l;\n\tcvt.f32.f16 %1, h;\n\t}"
        : "=f"(r.x), "=f"(r.y)
        : "r"(d));
    return r;
}

// Hi/lo split of four FP32 values in the packed operand layout (element e
// in bits 16 (e & 1) of word e >> 1): hi = round(v), lo = round(v - hi),
// both round-to-nearest in BF16 or FP16.  A BF16 value widens to FP32 by a
// 16-bit shift, so the BF16 form needs no conversion back.
template <bool BF16>
__device__ __forceinline__ void split4(const float4 v, uint2 &hi, uint2 &lo)
{
    if (BF16) {
        const uint32_t a = pack_bf16x2(v.x, v.y), b = pack_bf16x2(v.z, v.w);
        hi = make_uint2(a, b);
        lo = make_uint2(pack_bf16x2(v.x - __uint_as_float(a << 16), v.y - __uint_as_float(a & 0xffff0000u)),
                        pack_bf16x2(v.z - __uint_as_float(b << 16), v.w - __uint_as_float(b & 0xffff0000u)));
    } else {
        const uint32_t a = pack_f16x2(v.x, v.y), b = pack_f16x2(v.z, v.w);
        const float2 fa = unpack_f16x2(a), fb = unpack_f16x2(b);
        hi = make_uint2(a, b);
        lo = make_uint2(pack_f16x2(v.x - fa.x, v.y - fa.y), pack_f16x2(v.z - fb.x, v.w - fb.y));
    }
}

// BATCH = false: one query, its item read straight from the kernel's
// parameter space (constant-bank operands in the generator); BATCH = true:
// the item table in device memory, the current item staged in shared memory.
template <bool VAR, bool BATCH>
__global__ void __launch_bounds__(kTcThreads, 1) mc_tc_kernel(const __grid_constant__ TcBatch b)
{
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    // layout (dynamic): [Z hi: n_kt_max x 8 KB][Z lo: n_kt_max x 8 KB][stages x (hi 16 KB, lo 16 KB)]
    const PlainArgs &a = b.var; // VaR fields (single-item queries)
    unsigned char *base = (unsigned char *)(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    unsigned char *zhi = base;
    unsigned char *zlo = zhi + b.n_kt_max * kTcZBytes;
    unsigned char *lst = zlo + b.n_kt_max * kTcZBytes;

    __shared__ __align__(8) uint64_t full_bar[kTcStages], empty_bar[kTcStages], done_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ int sS[kTcPaths];
    __shared__ float sPort[kTcPaths];
    __shared__ int s_abort;
    __shared__ unsigned s_cons; // stages the MMA thread has consumed (for the abort drain)
    __shared__ long long s_unit;
    __shared__ unsigned long long sacc[4];
    __shared__ __align__(16) TcItem s_item; // BATCH: the current item
    int cur_item = -1;

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ncols = b.tmem_cols;

    if (tid < 4) sacc[tid] = 0ull;
    if (tid == 0) {
        for (int s = 0; s < kTcStages; s++) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&done_bar, 1);
        s_abort = 0;
        s_cons = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;

    int n_tail = 0;
    long long tail_fx = 0;
    // pipeline state (kept across tiles)
    unsigned prod_iter = 0, cons_iter = 0, tile_iter = 0;
    const long long total = b.dyn ? b.dyn[1] : b.total_tiles;
    const int n_items = b.dyn ? (int)b.dyn[0] : b.n_items;

    for (long long round = 0;; round++) {
        // claim a work unit: dynamic (atomic counter) for batches, static otherwise
        __syncthreads();
        if (tid == 0) s_unit = b.work ? (long long)atomicAdd(b.work, 1u) : blockIdx.x + round * gridDim.x;
        __syncthreads();
        const long long unit = s_unit;
        if (s_abort || unit * b.unit_tiles >= total) break;
        const long long tend = min(total, (unit + 1) * b.unit_tiles);
        for (long long tile = unit * b.unit_tiles; tile < tend; tile++, tile_iter++) {
            if (s_abort) break;
            // the item of this tile (items are ordered by tile_begin)
            if (BATCH) {
                int lo = 0, hi = n_items - 1;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (b.items[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
                }
                if (lo != cur_item) { // uniform: every thread computed the same index
                    const int *src = reinterpret_cast<const int *>(&b.items[lo]);
                    int *dst = reinterpret_cast<int *>(&s_item);
                    for (int w = tid; w < (int)(sizeof(TcItem) / 4); w += blockDim.x) dst[w] = src[w];
                    cur_item = lo;
                    __syncthreads();
                }
            }
            const TcItem &it = BATCH ? s_item : b.one;
            const int n = it.n, nq = (n + 3) >> 2, n_kt = it.n_kt, n_mt = it.n_mt;
            const long long p0 = (tile - it.tile_begin) * kTcPaths; // first path of the tile (item-local)
            // ---- 1. normals -> swizzled hi/lo Z tiles
            {
                const int p = tid & (kTcPaths - 1), r = tid >> 6; // kTcThreads / 64 threads per path
                const unsigned long long path = it.path0 + (unsigned long long)(p0 + p);
                const uint32_t plo = (uint32_t)path, phi = (uint32_t)(path >> 32);
                const int kq = n_kt * (kTcKt / 4);
                for (int q = r; q < kq; q += kTcThreads / kTcPaths) {
                    float z[4] = {0.f, 0.f, 0.f, 0.f};
                    if (q < nq) {
                        const int days = it.aggregated ? 1 : it.horizon;
                        for (int d = 0; d < days; d++) {
                            const uint4 wv = rg_philox(make_uint4((uint32_t)(d * nq + q), 0u, plo, phi), it.keys);
                            float z0, z1, z2, z3;
                            rg_box_muller_unscaled(wv.x, wv.y, z0, z1);
                            rg_box_muller_unscaled(wv.z, wv.w, z2, z3);
                            z[0] += z0;
                            z[1] += z1;
                            z[2] += z2;
                            z[3] += z3;
                        }
                        for (int e = 0; e < 4; e++) z[e] *= it.zscale;
                    }
                    uint2 hv, lv;
                    const float4 zv = make_float4(z[0], z[1], z[2], z[3]);
                    if (it.bf16) split4<true>(zv, hv, lv);
                    else split4<false>(zv, hv, lv);
                    const int k = 4 * q, kt = k / kTcKt, kk = k % kTcKt;
                    const uint32_t off = (uint32_t)kt * kTcZBytes + sw128_offset(p, kk);
                    *reinterpret_cast<uint2 *>(zhi + off) = hv;
                    *reinterpret_cast<uint2 *>(zlo + off) = lv;
                }
            }
            if (tid < kTcPaths) {
                sS[tid] = 0;
                sPort[tid] = 0.f;
            }
            fence_async_shared(); // generic-proxy writes of Z -> visible to the tensor cores
            tc_fence_before();
            __syncthreads();
            tc_fence_after();

            // ---- 2. producer (warp 1, one thread) and MMA issuer (warp 0, one thread)
            if (warp == 1 && lane == 0) {
                for (int mt = 0; mt < n_mt; mt++) {
                    const int kend = min(n_kt, (kTcRows * (mt + 1) + kTcKt - 1) / kTcKt);
                    const int kts = (mt == n_mt - 1) ? n_kt : kend;
                    for (int kt = 0; kt < kts; kt++, prod_iter++) {
                        const int s = prod_iter % kTcStages;
                        const unsigned ph = ((prod_iter / kTcStages) & 1u) ^ 1u;
                        if (!mbar_wait(&empty_bar[s], ph)) {
                            atomicOr(b.err, 1u);
                            s_abort = 1;
                            break;
                        }
                        if (b.inject_stall && prod_iter == 1) continue; // never filled: the consumer's wait runs out
                        mbar_expect_tx(&full_bar[s], 2 * kTcTileBytes);
                        const unsigned char *src = it.tiles + ((size_t)(mt * n_kt + kt) * 2) * kTcTileBytes;
                        unsigned char *dst = lst + (size_t)s * 2 * kTcTileBytes;
                        bulk_copy(dst, src, kTcTileBytes, &full_bar[s]);
                        bulk_copy(dst + kTcTileBytes, src + kTcTileBytes, kTcTileBytes, &full_bar[s]);
                    }
                    if (s_abort) break;
                }
            } else if (warp == 0 && lane == 0) {
                const uint32_t idesc = tc_idesc(it.bf16, kTcRows, kTcPaths);
                for (int mt = 0; mt < n_mt; mt++) {
                    const int kend = min(n_kt, (kTcRows * (mt + 1) + kTcKt - 1) / kTcKt);
                    const int kts = (mt == n_mt - 1) ? n_kt : kend;
                    const uint32_t d_tmem = tmem + (uint32_t)(mt * kTcPaths);
                    for (int kt = 0; kt < kts; kt++, cons_iter++) {
                        const int s = cons_iter % kTcStages;
                        const unsigned ph = (cons_iter / kTcStages) & 1u;
                        if (s_abort || !mbar_wait(&full_bar[s], ph)) {
                            atomicOr(b.err, 2u);
                            s_abort = 1;
                            break;
                        }
                        tc_fence_after();
                        const uint32_t lhi = smem_u32(lst + (size_t)s * 2 * kTcTileBytes);
                        const uint32_t llo = lhi + kTcTileBytes;
                        const uint32_t zh = smem_u32(zhi + (size_t)kt * kTcZBytes);
                        const uint32_t zl = smem_u32(zlo + (size_t)kt * kTcZBytes);
#pragma unroll
                        for (int ks = 0; ks < kTcKt / 16; ks++) {
                            const uint32_t o = (uint32_t)ks * 32; // 16 elements = 32 bytes along K
                            const uint32_t acc0 = (kt > 0 || ks > 0) ? 1u : 0u;
                            tc_mma(d_tmem, sw128_desc(lhi + o), sw128_desc(zh + o), idesc, acc0);
                            tc_mma(d_tmem, sw128_desc(lhi + o), sw128_desc(zl + o), idesc, 1u);
                            tc_mma(d_tmem, sw128_desc(llo + o), sw128_desc(zh + o), idesc, 1u);
                        }
                        tc_commit(&empty_bar[s]); // stage free once these MMAs complete
                    }
                    if (s_abort) break;
                }
                tc_commit(&done_bar); // all MMAs of the tile issued so far
                s_cons = cons_iter;
            }
            // lanes 1-31 of warps 0 and 1 wait here, blocked, for their lane 0:
            // spinning on done_bar beside it would take its issue slots
            __syncwarp();
            // ---- 3. epilogue
            const bool done_ok = mbar_wait(&done_bar, tile_iter & 1u);
            if (!done_ok && tid == 0) {
                atomicOr(b.err, 4u);
                s_abort = 1;
            }
            tc_fence_after();
            if (done_ok && !s_abort) {
                constexpr int kGroups = kTcThreads / 128;          // column groups
                constexpr int kCols = kTcPaths / kGroups;          // columns per warp
                const int quarter = warp & 3, sub = warp >> 2;     // lanes 32*quarter.., columns kCols*sub..
                for (int mt = 0; mt < n_mt; mt++) {
                    const int row = mt * kTcRows + quarter * 32 + lane; // this thread's asset row
                    const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(mt * kTcPaths + sub * kCols);
                    uint32_t v[kCols];
                    static_assert(kCols == 8 || kCols == 16, "epilogue load shape");
                    if constexpr (kCols == 16) {
                        asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                                     "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                                       "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                                       "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                                     : "r"(taddr));
                    } else {
                        asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                                     : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                                       "=r"(v[6]), "=r"(v[7])
                                     : "r"(taddr));
                    }
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    // threshold on the scaled accumulator: D/2^8 < -x - H mu_i
                    const bool asset = row < n;
                    const float thr = asset ? tc_threshold(it, row) : 0.f;
                    int cnt = 0;
#pragma unroll
                    for (int c = 0; c < kCols; c++) {
                        const float d = __uint_as_float(v[c]);
                        const unsigned m = __ballot_sync(0xffffffffu, asset && d < thr);
                        if (lane == c) cnt = __popc(m);
                    }
                    if (lane < kCols && cnt) atomicAdd(&sS[sub * kCols + lane], cnt);
                    if (row == n) {
#pragma unroll
                        for (int c = 0; c < kCols; c++)
                            sPort[sub * kCols + c] = it.hwmu_f + __uint_as_float(v[c]) * (1.0f / kTcLScale);
                    }
                }
            }
            tc_fence_before();
            __syncthreads();
            if (!s_abort && tid < kTcPaths) {
                const long long p = p0 + tid;
                const bool live = p < it.n_paths;
                int crash = 0, breach = 0;
                if (live) {
                    const int S = sS[tid];
                    const float port = sPort[tid];
                    crash = (S >= it.k) ? 1 : 0;
                    breach = (it.has_w && port < it.port_thr) ? 1 : 0;
                    if (it.s_values) it.s_values[p] = S;
                    if (it.port_values) it.port_values[p] = port;
                    if (VAR) var_path(a, port, nullptr, n_tail, tail_fx); // histogram pass: global atomics
                }
                crash = __reduce_add_sync(0xffffffffu, crash);
                breach = __reduce_add_sync(0xffffffffu, breach);
                if (lane == 0) {
                    if (crash) atomicAdd(&it.counts[0], (unsigned long long)crash);
                    if (breach) atomicAdd(&it.counts[1], (unsigned long long)breach);
                }
            }
            __syncthreads();
            tc_fence_after();
        }
    }

    // ---- teardown: drain in-flight copies and MMAs (bounded), free TMEM
    if (s_abort) {
        if (warp == 0 && lane == 0) {
            tc_commit(&done_bar);
            mbar_wait(&done_bar, tile_iter & 1u);
        }
        if (warp == 1 && lane == 0) {
            // copies issued but not consumed: wait for them to land
            for (unsigned i = s_cons; i < prod_iter; i++)
                mbar_wait(&full_bar[i % kTcStages], (i / kTcStages) & 1u);
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
    if (VAR) cta_flush(a, 0, 0, n_tail, tail_fx, sacc, nullptr, true);
}

// ----------------------------------------------------------------------
// Warp-specialised form of the same computation.  1024 threads:
//   warps 0-3    epilogue: warp w reads TMEM lanes 32 w .. +31 of a row tile
//                as soon as that row tile is fully accumulated;
//   warp 4       lane 0 issues the MMAs and, unless SPLIT, streams the Lhat
//                tiles into the ring (bulk copies issued between MMA pairs
//                whenever a stage is free);
//   warp 5       SPLIT: lane 0 streams the Lhat tiles (used when the MMAs
//                bound the kernel, so refills never wait for the MMA thread)
//   warps 5|6-31 (864 | 832 threads) generator: draws the normals one
//                64-column K tile at a time into a ring of K-tile slots, a
//                thread drawing one path's two adjacent quads at a time.
// The MMAs run K-tile-outer (for each K tile, every row tile that needs it),
// so a K tile is needed only while its MMAs run: K tiles are numbered in
// order across the CTA's path tiles (g), K tile g lives in slot g % kZSlots
// and the slot is released (zempty) as soon as its MMAs complete; a few
// slots instead of a whole path tile's normals leave room for a 4-5 stage
// Lhat ring, which hides the L2 latency of the copies.  Row tile m is
// complete after K tile kts(m) - 1 (lower triangle), so its epilogue runs
// while later K tiles are still being drawn, and the next tile's MMAs
// overwrite its accumulator once the epilogue has read it (acc_free): only
// the last row tile's epilogue is on the critical path.
// Barriers (all waits bounded):
//   tile_pub[s]  generator -> other roles: tile index and item of slot s
//   zfull[z]     generator -> MMA: the K tile in slot z written (one arrival
//                per generator thread)
//   zempty[z]    MMA -> generator: the MMAs that read slot z are complete
//   full/empty   Lhat ring (copy completion, MMA completion)
//   acc_full[m]  MMA -> epilogue: row tile m of the tile accumulated
//   acc_free[m]  epilogue -> MMA: row tile m read (one arrival per warp)
//   slot_free[s] epilogue -> generator: the tile in slot s is finished
// The K-tile number g, use counts per row tile and per item slot (the same
// on both sides of each barrier) give the phase parities, since items of a
// batch differ in size.  The tile index is read after tile_pub, never after
// zfull[0]: slot s is republished only after the epilogue finished the tile
// that used it, so no waiter can fall a whole phase behind.
static constexpr int kWsThreads = 1024;
static constexpr int kWsEpiWarps = 4;
static constexpr int kWsMmaWarp = 4;
static constexpr int kTcMaxMt = (kTcMaxKt * kTcKt + 1 + kTcRows - 1) / kTcRows;
// Paths per tile P (the MMA's N): the widest of 128, 96, 64 at which the
// item's row tiles fit in tensor memory (n_mt x P <= 512 columns: P = 128 up
// to N = 511, 96 up to N = 639).  A wider tile moves fewer operand bytes per
// MMA flop (7 KB per 1.5x the work of a 64-path MMA at P = 96, 8 KB per 2x
// at 128), streams each Lhat tile once per P paths and issues fewer MMAs per
// path.  Shared memory: Z ring (kZSlots K-tile slots, hi + lo) + Lhat ring
// (kStages x 32 KB) + alignment = 230.4 KB for every P.
template <int P> struct WsShape {
    static constexpr int kZBytes = P * kTcKt * 2;          // one part of a Z K tile
    static constexpr int kZSlots = (P == 128) ? 3 : 4;     // K-tile slots of Z
    static constexpr int kStages = (P == 64) ? 5 : 4;      // Lhat ring stages (hi + lo, 32 KB each)
    static constexpr size_t kSmem = 1024 + (size_t)kZSlots * 2 * kZBytes + (size_t)kStages * 2 * kTcTileBytes;
    static_assert(P % 16 == 0 && P >= 64 && P <= 128, "path tile");
    static_assert(kSmem <= 227 * 1024 - 2048, "shared memory");
};

__device__ __forceinline__ void named_sync(int id, int n)
{
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(n) : "memory");
}

// named barrier that also ORs a predicate over the participating threads
__device__ __forceinline__ int named_sync_or(int id, int n, int pred)
{
    int r;
    asm volatile("{\n\t.reg .pred p, q;\n\tsetp.ne.s32 p, %1, 0;\n\tbar.red.or.pred q, %2, %3, p;\n\t"
                 "selp.s32 %0, 1, 0, q;\n\t}"
                 : "=r"(r)
                 : "r"(pred), "r"(id), "r"(n)
                 : "memory");
    return r;
}

// K tiles that row tile mt needs (lower triangle; the last row tile also
// holds the portfolio row w^T L, which spans every column)
__device__ __forceinline__ int tc_kts(int mt, int n_mt, int n_kt)
{
    return (mt == n_mt - 1) ? n_kt : min(n_kt, (kTcRows * (mt + 1) + kTcKt - 1) / kTcKt);
}

template <bool VAR, bool BATCH, int P, bool SPLIT>
__global__ void __launch_bounds__(kWsThreads, 1) mc_tcws_kernel(const __grid_constant__ TcBatch b)
{
    using Sh = WsShape<P>;
    constexpr int kStages = Sh::kStages, kZB = Sh::kZBytes, kWsZSlots = Sh::kZSlots;
    // SPLIT: warp 5 streams the Lhat tiles (when the MMAs bound the kernel,
    // refills never wait for the MMA thread); otherwise the MMA thread
    // issues the copies too and warp 5 draws normals
    constexpr int kWsGenWarp0 = SPLIT ? 6 : 5;
    constexpr int kWsGenThreads = kWsThreads - 32 * kWsGenWarp0;
    extern __shared__ __align__(1024) unsigned char tc_smem[];
    const PlainArgs &a = b.var;
    unsigned char *base = (unsigned char *)(((uintptr_t)tc_smem + 1023) & ~(uintptr_t)1023);
    unsigned char *zhi = base;
    unsigned char *zlo = zhi + kWsZSlots * kZB;
    unsigned char *lst = zlo + kWsZSlots * kZB;

    __shared__ __align__(8) uint64_t full_bar[kStages], empty_bar[kStages];
    __shared__ __align__(8) uint64_t zfull[kWsZSlots], zempty[kWsZSlots];
    __shared__ __align__(8) uint64_t acc_full[kTcMaxMt], acc_free[kTcMaxMt];
    __shared__ __align__(8) uint64_t tile_pub[2], slot_free[2], drain_bar;
    __shared__ uint32_t tmem_base_sh;
    __shared__ int sS[P];
    __shared__ float sPort[P];
    // set by a role whose bounded wait ran out; the others then make no
    // further waits and finish
    __shared__ int tm_abort;
    __shared__ long long s_tile[2];
    __shared__ long long s_unit;
    __shared__ unsigned long long sacc[4];
    __shared__ __align__(16) TcItem s_item[BATCH ? 2 : 1];

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int ncols = b.tmem_cols;
    if (tid < 4) sacc[tid] = 0ull;
    if (tid < P) {
        sS[tid] = 0;
        sPort[tid] = 0.f;
    }
    if (tid == 0) {
        for (int s = 0; s < kStages; s++) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        for (int z = 0; z < kWsZSlots; z++) {
            mbar_init(&zfull[z], kWsGenThreads);
            mbar_init(&zempty[z], 1);
        }
        for (int m = 0; m < kTcMaxMt; m++) {
            mbar_init(&acc_full[m], 1);
            mbar_init(&acc_free[m], kWsEpiWarps);
        }
        for (int s = 0; s < 2; s++) {
            mbar_init(&tile_pub[s], 1);
            mbar_init(&slot_free[s], 1);
        }
        mbar_init(&drain_bar, 1);
        tm_abort = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base_sh)),
                     "r"(ncols));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base_sh;
    const long long total = b.dyn ? b.dyn[1] : b.total_tiles;
    const int n_items = b.dyn ? (int)b.dyn[0] : b.n_items;
    int n_tail = 0;
    long long tail_fx = 0;

    if (warp >= kWsGenWarp0) {
        // ======================= generator =======================
        // gab: this thread's abort flag.  Generator threads do not meet at
        // K-tile boundaries, so a timeout is first local; the reduction
        // barrier at the start of each tile makes it uniform before any
        // decision that changes barrier participation.
        const int gtid = tid - 32 * kWsGenWarp0;
        unsigned g0 = 0; // K tiles of the previous path tiles
        int gab = 0;
        long long unit = -1, unit_end = 0, next_static = blockIdx.x;
        for (unsigned j = 0;; j++) {
            const int slot = j & 1;
            // the slot must be free (epilogue of tile j-2 done); after an
            // abort on either side no wait is made
            if (!gab && !tm_abort && !mbar_wait(&slot_free[slot], ((j >> 1) & 1u) ^ 1u)) {
                atomicOr(b.err, 8u);
                gab = 1;
            }
            gab = named_sync_or(2, kWsGenThreads, gab);
            if (gtid == 0) {
                long long tile = -1;
                if (!gab && !tm_abort) {
                    if (b.work) {
                        if (unit < 0 || unit_end <= 0) {
                            unit = (long long)atomicAdd(b.work, 1u);
                            unit_end = b.unit_tiles;
                        }
                        tile = unit * b.unit_tiles + (b.unit_tiles - unit_end);
                        unit_end--;
                        if (tile >= total || unit * b.unit_tiles >= total) tile = -1;
                    } else {
                        tile = next_static;
                        next_static += gridDim.x;
                        if (tile >= total) tile = -1;
                    }
                }
                s_tile[slot] = tile;
                if (BATCH && tile >= 0) {
                    int lo = 0, hi = n_items - 1;
                    while (lo < hi) {
                        const int mid = (lo + hi + 1) >> 1;
                        if (b.items[mid].tile_begin <= tile) lo = mid; else hi = mid - 1;
                    }
                    s_unit = lo;
                }
            }
            named_sync(2, kWsGenThreads);
            const long long tile = s_tile[slot];
            if (BATCH && tile >= 0) { // stage the item in its slot
                const int *src = reinterpret_cast<const int *>(&b.items[s_unit]);
                int *dst = reinterpret_cast<int *>(&s_item[slot]);
                for (int w = gtid; w < (int)(sizeof(TcItem) / 4); w += kWsGenThreads) dst[w] = src[w];
                named_sync(2, kWsGenThreads);
            }
            // publish the tile (or the end, -1) to the other roles
            if (gtid == 0) mbar_arrive(&tile_pub[slot]);
            if (tile < 0) break; // uniform: every thread read the same s_tile
            const TcItem &it = BATCH ? s_item[slot] : b.one;
            const int n = it.n, nq = (n + 3) >> 2, n_kt = it.n_kt;
            const long long p0 = (tile - it.tile_begin) * P;
            // each thread walks its items of the tile in K-tile order and
            // arrives on zfull[kt] once it has written its share of kt (no
            // group barrier, so no thread idles at K-tile boundaries)
            for (int kt = 0; kt < n_kt; kt++) {
                const unsigned g = g0 + (unsigned)kt;
                const int zs = (int)(g % kWsZSlots);
                // the MMAs on the slot's previous K tile (g - kWsZSlots) are done
                if (!gab && !tm_abort && !mbar_wait(&zempty[zs], ((g / kWsZSlots) & 1u) ^ 1u)) {
                    atomicOr(b.err, 16u);
                    gab = 1;
                }
                // an item is one path's pair of adjacent quads (8 K columns,
                // one 16-byte chunk of the swizzled Z row); items of kt are
                // i = kt*per_kt + local, assigned round robin over the whole
                // tile (i % kWsGenThreads == gtid)
                const int per_kt = P * (kTcKt / 8);
                int first = gtid - (kt * per_kt) % kWsGenThreads;
                if (first < 0) first += kWsGenThreads;
                const int days = it.aggregated ? 1 : it.horizon;
                for (int item = first; item < per_kt; item += kWsGenThreads) {
                    const int qp = item / P, p = item - qp * P, q = kt * (kTcKt / 4) + 2 * qp;
                    const unsigned long long path = it.path0 + (unsigned long long)(p0 + p);
                    const uint32_t plo = (uint32_t)path, phi = (uint32_t)(path >> 32);
                    // the two quads' Philox rounds interleaved when both are real
                    float4 z = make_float4(0.f, 0.f, 0.f, 0.f), y = make_float4(0.f, 0.f, 0.f, 0.f);
                    if (q + 1 < nq) tc_quad_sum2(q, plo, phi, q + 1, plo, phi, nq, days, it.keys, z, y);
                    else if (q < nq) z = tc_quad_sum(q, nq, days, plo, phi, it.keys);
                    z.x *= it.zscale;
                    z.y *= it.zscale;
                    z.z *= it.zscale;
                    z.w *= it.zscale;
                    y.x *= it.zscale;
                    y.y *= it.zscale;
                    y.z *= it.zscale;
                    y.w *= it.zscale;
                    uint2 hz, lz, hy, ly;
                    if (it.bf16) {
                        split4<true>(z, hz, lz);
                        split4<true>(y, hy, ly);
                    } else {
                        split4<false>(z, hz, lz);
                        split4<false>(y, hy, ly);
                    }
                    // padding quads (q >= nq) store zeros
                    const uint32_t off = (uint32_t)zs * kZB + sw128_offset(p, 8 * qp);
                    *reinterpret_cast<uint4 *>(zhi + off) = make_uint4(hz.x, hz.y, hy.x, hy.y);
                    *reinterpret_cast<uint4 *>(zlo + off) = make_uint4(lz.x, lz.y, ly.x, ly.y);
                }
                fence_async_shared(); // this thread's writes -> async proxy (tensor cores)
                mbar_arrive(&zfull[zs]);
            }
            g0 += (unsigned)n_kt;
        }
    } else if (SPLIT && warp == kWsMmaWarp + 1) {
        // ======================= Lhat producer =======================
        if (lane == 0) {
            unsigned prod_iter = 0;
            int skipped = -1; // the stage left unfilled by the fault injection
            for (unsigned j = 0; !tm_abort; j++) {
                const int slot = j & 1;
                if (!mbar_wait(&tile_pub[slot], (j >> 1) & 1u)) {
                    atomicOr(b.err, 32u);
                    tm_abort = 1;
                    break;
                }
                if (s_tile[slot] < 0) break;
                const TcItem &it = BATCH ? s_item[slot] : b.one;
                const int n_kt = it.n_kt, n_mt = it.n_mt;
                for (int kt = 0; kt < n_kt && !tm_abort; kt++) {
                    for (int mt = 0; mt < n_mt; mt++) {
                        if (kt >= tc_kts(mt, n_mt, n_kt)) continue;
                        const int s = prod_iter % kStages;
                        if (tm_abort || !mbar_wait(&empty_bar[s], ((prod_iter / kStages) & 1u) ^ 1u)) {
                            atomicOr(b.err, 1u);
                            tm_abort = 1;
                            break;
                        }
                        if (b.inject_stall && prod_iter == 1) { // never filled: the consumer's wait runs out
                            skipped = (int)prod_iter++;
                            continue;
                        }
                        mbar_expect_tx(&full_bar[s], 2 * kTcTileBytes);
                        const unsigned char *src = it.tiles + ((size_t)(mt * n_kt + kt) * 2) * kTcTileBytes;
                        unsigned char *dst = lst + (size_t)s * 2 * kTcTileBytes;
                        bulk_copy(dst, src, kTcTileBytes, &full_bar[s]);
                        bulk_copy(dst + kTcTileBytes, src + kTcTileBytes, kTcTileBytes, &full_bar[s]);
                        prod_iter++;
                    }
                }
            }
            // the copies still in flight land before the kernel ends
            for (unsigned i = prod_iter > kStages ? prod_iter - kStages : 0; i < prod_iter; i++)
                if ((int)i != skipped) mbar_wait(&full_bar[i % kStages], (i / kStages) & 1u);
        }
        __syncwarp();
    } else if (warp == kWsMmaWarp) {
        // ============ MMA issue (and, unless SPLIT, the Lhat copies) ============
        // Pairs (row tile, K tile) are numbered in consumption order across
        // tiles: pi copies issued, ci pairs multiplied.  pump() issues copies
        // while the ring has room, probing its barriers without blocking; it
        // blocks only when the next pair to multiply has no copy yet (need).
        // The copy cursor enters a tile only once that tile is published.
        if (lane == 0) {
            unsigned pi = 0, ci = 0;
            int skipped = -1;             // the pair left unfilled by the fault injection
            unsigned pj = 0;              // tile (sequence number) of the copy cursor
            bool p_live = false, p_end = false;
            int pkt = 0, pmt = 0, p_nkt = 0, p_nmt = 0;
            const unsigned char *p_tiles = nullptr;
            auto pump = [&](bool need) -> bool {
                while (!p_end && pi < ci + kStages) {
                    const bool must = need && pi == ci;
                    if (!p_live) {
                        const int ps = (int)(pj & 1u);
                        const unsigned par = (pj >> 1) & 1u;
                        if (!mbar_test(&tile_pub[ps], par)) {
                            if (!must) return true;
                            if (!mbar_wait(&tile_pub[ps], par)) return false;
                        }
                        if (s_tile[ps] < 0) {
                            p_end = true;
                            return true;
                        }
                        const TcItem &pit = BATCH ? s_item[ps] : b.one;
                        p_nkt = pit.n_kt;
                        p_nmt = pit.n_mt;
                        p_tiles = pit.tiles;
                        pkt = 0;
                        pmt = 0; // (K tile 0, row tile 0) is always a pair
                        p_live = true;
                    }
                    const int st = (int)(pi % kStages);
                    const unsigned eph = ((pi / kStages) & 1u) ^ 1u;
                    if (!mbar_test(&empty_bar[st], eph)) {
                        if (!must) return true;
                        if (!mbar_wait(&empty_bar[st], eph)) return false;
                    }
                    if (b.inject_stall && pi == 1) { // never filled: the MMA side's wait runs out
                        skipped = (int)pi;
                    } else {
                        mbar_expect_tx(&full_bar[st], 2 * kTcTileBytes);
                        const unsigned char *src = p_tiles + ((size_t)(pmt * p_nkt + pkt) * 2) * kTcTileBytes;
                        unsigned char *dst = lst + (size_t)st * 2 * kTcTileBytes;
                        bulk_copy(dst, src, kTcTileBytes, &full_bar[st]);
                        bulk_copy(dst + kTcTileBytes, src + kTcTileBytes, kTcTileBytes, &full_bar[st]);
                    }
                    pi++;
                    // next pair: row tiles that need K tile pkt form a suffix of 0..n_mt-1
                    do {
                        if (++pmt == p_nmt) {
                            pmt = 0;
                            ++pkt;
                        }
                    } while (pkt < p_nkt && pkt >= tc_kts(pmt, p_nmt, p_nkt));
                    if (pkt == p_nkt) {
                        p_live = false;
                        pj++;
                    }
                }
                return true;
            };

            unsigned g0 = 0, fpar = 0; // fpar bit m: parity of the uses of row tile m
            unsigned rs = 0, rph = 0;  // Lhat ring: stage and phase parity of pair ci
            const uint32_t lst_lo = sw128_desc_lo(smem_u32(lst));
            for (unsigned j = 0; !tm_abort; j++) {
                const int slot = j & 1;
                if (!mbar_wait(&tile_pub[slot], (j >> 1) & 1u)) {
                    atomicOr(b.err, 32u);
                    tm_abort = 1;
                    break;
                }
                if (s_tile[slot] < 0) break;
                const TcItem &it = BATCH ? s_item[slot] : b.one;
                const int n_kt = it.n_kt, n_mt = it.n_mt;
                const uint32_t idesc = tc_idesc(it.bf16, kTcRows, P);
                for (int kt = 0; kt < n_kt && !tm_abort; kt++) {
                    const unsigned g = g0 + (unsigned)kt;
                    const int zs = (int)(g % kWsZSlots);
                    if ((!SPLIT && !pump(false)) || !mbar_wait(&zfull[zs], (g / kWsZSlots) & 1u)) {
                        atomicOr(b.err, 64u);
                        tm_abort = 1;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t zh_lo = sw128_desc_lo(smem_u32(zhi + (size_t)zs * kZB));
                    const uint32_t zl_lo = sw128_desc_lo(smem_u32(zlo + (size_t)zs * kZB));
                    for (int mt = 0; mt < n_mt; mt++) {
                        const int kts = tc_kts(mt, n_mt, n_kt);
                        if (kt >= kts) continue;
                        // the first write to row tile mt: the epilogue has read the previous tile's
                        if (kt == 0 && !mbar_wait(&acc_free[mt], ((fpar >> mt) & 1u) ^ 1u)) {
                            atomicOr(b.err, 128u);
                            tm_abort = 1;
                            break;
                        }
                        if (!SPLIT && !pump(true)) {
                            atomicOr(b.err, 1u);
                            tm_abort = 1;
                            break;
                        }
                        if (!mbar_wait(&full_bar[rs], rph)) {
                            atomicOr(b.err, 2u);
                            tm_abort = 1;
                            break;
                        }
                        tc_fence_after();
                        tc_mma_pair(tmem + (uint32_t)(mt * P), lst_lo + (uint32_t)rs * (2 * kTcTileBytes >> 4),
                                    zh_lo, zl_lo, idesc, kt > 0 ? 1u : 0u);
                        tc_commit(&empty_bar[rs]);
                        ci++;
                        if (++rs == kStages) {
                            rs = 0;
                            rph ^= 1u;
                        }
                        if (kt == kts - 1) tc_commit(&acc_full[mt]); // row tile mt complete
                    }
                    tc_commit(&zempty[zs]); // the slot may be overwritten once these MMAs complete
                }
                g0 += (unsigned)n_kt;
                fpar ^= (1u << n_mt) - 1u;
            }
            // copies issued but not multiplied (only after an abort) land
            // before the kernel ends; every MMA issued (and every commit's
            // arrival) completes before the tensor memory and the barriers
            // are released
            if (!SPLIT)
                for (unsigned i = ci; i < pi; i++)
                    if ((int)i != skipped) mbar_wait(&full_bar[i % kStages], (i / kStages) & 1u);
            tc_commit(&drain_bar);
            mbar_wait(&drain_bar, 0u);
        }
        __syncwarp();
    } else {
        // ======================= epilogue (warps 0-3) =======================
        unsigned apar = 0; // bit m: parity of the uses of row tile m
        for (unsigned j = 0;; j++) {
            const int slot = j & 1;
            int ab = 0;
            if (!tm_abort && !mbar_wait(&tile_pub[slot], (j >> 1) & 1u)) {
                atomicOr(b.err, 32u);
                ab = 1;
            }
            if (named_sync_or(1, 32 * kWsEpiWarps, ab || tm_abort)) { // uniform over the four warps
                tm_abort = 1;
                break;
            }
            const long long tile = s_tile[slot];
            if (tile < 0) break;
            const TcItem &it = BATCH ? s_item[slot] : b.one;
            const int n = it.n, n_mt = it.n_mt;
            bool dead = false;
            for (int mt = 0; mt < n_mt; mt++) {
                int wab = 0;
                if (!tm_abort && !mbar_wait(&acc_full[mt], (apar >> mt) & 1u)) {
                    atomicOr(b.err, 4u);
                    wab = 1;
                }
                if (named_sync_or(1, 32 * kWsEpiWarps, wab || tm_abort)) {
                    dead = true;
                    break;
                }
                tc_fence_after();
                const int row = mt * kTcRows + warp * 32 + lane;
                const bool asset = row < n;
                const float thr = asset ? tc_threshold(it, row) : 0.f;
#pragma unroll
                for (int cb = 0; cb < P / 16; cb++) {
                    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(mt * P + cb * 16);
                    uint32_t v[16];
                    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                                 "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                                 : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]),
                                   "=r"(v[6]), "=r"(v[7]), "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]),
                                   "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
                                 : "r"(taddr));
                    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
                    int cnt = 0;
#pragma unroll
                    for (int c = 0; c < 16; c++) {
                        const unsigned m = __ballot_sync(0xffffffffu, asset && __uint_as_float(v[c]) < thr);
                        if (lane == c) cnt = __popc(m);
                    }
                    if (lane < 16 && cnt) atomicAdd(&sS[cb * 16 + lane], cnt);
                    if (row == n) {
#pragma unroll
                        for (int c = 0; c < 16; c++)
                            sPort[cb * 16 + c] = it.hwmu_f + __uint_as_float(v[c]) * (1.0f / kTcLScale);
                    }
                }
                // this warp's reads of row tile mt are complete: the next tile may overwrite it
                tc_fence_before();
                __syncwarp();
                if (lane == 0) mbar_arrive(&acc_free[mt]);
            }
            if (dead) {
                tm_abort = 1;
                break;
            }
            apar ^= (1u << n_mt) - 1u;
            named_sync(1, 32 * kWsEpiWarps); // every count of the tile is in sS / sPort
            if (tid < P) {
                const long long p = (tile - it.tile_begin) * P + tid;
                int crash = 0, breach = 0;
                if (p < it.n_paths) {
                    const int S = sS[tid];
                    const float port = sPort[tid];
                    crash = (S >= it.k) ? 1 : 0;
                    breach = (it.has_w && port < it.port_thr) ? 1 : 0;
                    if (it.s_values) it.s_values[p] = S;
                    if (it.port_values) it.port_values[p] = port;
                    if (VAR) var_path(a, port, nullptr, n_tail, tail_fx);
                }
                crash = __reduce_add_sync(0xffffffffu, crash);
                breach = __reduce_add_sync(0xffffffffu, breach);
                if (lane == 0) {
                    if (crash) atomicAdd(&it.counts[0], (unsigned long long)crash);
                    if (breach) atomicAdd(&it.counts[1], (unsigned long long)breach);
                }
                sS[tid] = 0;
                sPort[tid] = 0.f;
            }
            named_sync(1, 32 * kWsEpiWarps); // resets done before the next tile's counts
            if (tid == 0) mbar_arrive(&slot_free[slot]); // the generator may reuse this slot
        }
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
    if (VAR) cta_flush(a, 0, 0, n_tail, tail_fx, sacc, nullptr, true);
}

// Pre-swizzled Lhat tiles: rows 0..N-1 = L (lower triangle), row N = w^T L,
// scaled by 2^8, split into hi and lo (FP16 or BF16), each (row tile, K tile)
// block laid out exactly as the kernel's shared memory expects.
__global__ void build_tc_tiles_kernel(const double *L, const float *w, int n, int n_mt, int n_kt, int bf16,
                                      unsigned char *tiles)
{
    const long long total = (long long)n_mt * kTcRows * n_kt * kTcKt;
    for (long long idx = blockIdx.x * (long long)blockDim.x + threadIdx.x; idx < total;
         idx += (long long)gridDim.x * blockDim.x) {
        const int col = (int)(idx % (n_kt * kTcKt));
        const int row = (int)(idx / (n_kt * kTcKt));
        double v = 0.0;
        if (col < n) {
            if (row < n) {
                if (col <= row) v = L[(long long)row * n + col];
            } else if (row == n) {
                for (int i = col; i < n; i++) v += (double)w[i] * L[(long long)i * n + col];
            }
        }
        const float f = (float)(v * kTcLScale);
        unsigned short hi, lo;
        if (bf16) {
            const __nv_bfloat16 h = __float2bfloat16_rn(f);
            hi = __bfloat16_as_ushort(h);
            lo = __bfloat16_as_ushort(__float2bfloat16_rn(f - __bfloat162float(h)));
        } else {
            const __half h = __float2half_rn(f);
            hi = __half_as_ushort(h);
            lo = __half_as_ushort(__float2half_rn(f - __half2float(h)));
        }
        const int mt = row / kTcRows, r = row % kTcRows, kt = col / kTcKt, k = col % kTcKt;
        const size_t blk = ((size_t)(mt * n_kt + kt) * 2) * kTcTileBytes;
        const uint32_t off = sw128_offset(r, k);
        *reinterpret_cast<unsigned short *>(tiles + blk + off) = hi;
        *reinterpret_cast<unsigned short *>(tiles + blk + kTcTileBytes + off) = lo;
    }
}

int tc_max_n() { return kTcMaxKt * kTcKt; }
int tc_max_k_tiles() { return kTcMaxKt; }
static int tc_row_tiles(int n) { return (n + 1 + kTcRows - 1) / kTcRows; }
static int tc_k_tiles(int n) { return (n + kTcKt - 1) / kTcKt; }
size_t tc_tile_bytes(int n) { return (size_t)tc_row_tiles(n) * tc_k_tiles(n) * 2 * kTcTileBytes; }

cudaError_t launch_build_tc_tiles(const double *L64, const float *w32, int n, int bf16, unsigned char *tiles,
                                  cudaStream_t s)
{
    build_tc_tiles_kernel<<<256, 256, 0, s>>>(L64, w32, n, tc_row_tiles(n), tc_k_tiles(n), bf16, tiles);
    return cudaGetLastError();
}

static int tmem_cols_for(int n_mt, int paths)
{
    int c = 32;
    while (c < n_mt * paths) c <<= 1;
    return c;
}

static size_t tc_smem_bytes(int n_kt_max)
{
    return 1024 + (size_t)n_kt_max * 2 * kTcZBytes + (size_t)kTcStages * 2 * kTcTileBytes;
}

// Paths per tile of the warp-specialised kernel for items of at most
// n_mt_max row tiles (tensor memory holds n_mt x paths FP32 columns).
int tc_batch_paths(int n_mt_max) { return n_mt_max * 128 <= 512 ? 128 : (n_mt_max * 96 <= 512 ? 96 : 64); }

static void fill_item(TcItem &it, const PlainArgs &a, const unsigned char *tiles, int bf16, bool aggregated,
                      double wmu, long long tile_begin)
{
    memset(&it, 0, sizeof(it));
    it.tiles = tiles;
    it.mu64 = a.mu64;
    it.counts = a.counts;
    it.s_values = a.s_values;
    it.port_values = a.port_values;
    it.path0 = a.path0;
    it.n_paths = a.n_paths;
    it.tile_begin = tile_begin;
    it.keys = a.keys;
    it.hwmu = (double)a.horizon * wmu;
    it.hwmu_f = (float)it.hwmu;
    it.n = a.n;
    it.n_mt = tc_row_tiles(a.n);
    it.n_kt = tc_k_tiles(a.n);
    it.horizon = a.horizon;
    it.k = a.k;
    it.has_w = a.has_w;
    it.aggregated = aggregated ? 1 : 0;
    it.bf16 = bf16;
    it.neg_x = a.neg_x;
    it.port_thr = a.port_thr;
    it.zscale = (float)((double)kBmScale * (aggregated ? std::sqrt((double)a.horizon) : 1.0));
}

template <class K>
static cudaError_t launch_one(K kern, const TcBatch &b, int threads, size_t smem, long long grid, cudaStream_t s)
{
    cudaError_t e = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
    kern<<<(unsigned)grid, threads, smem, s>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_tc(const PlainArgs &a, const unsigned char *tiles, int bf16, bool aggregated, double wmu,
                      unsigned int *err, bool inject_stall, int sm_count, cudaStream_t s)
{
    if (a.n > tc_max_n()) return cudaErrorInvalidValue;
    TcBatch b;
    memset(&b, 0, sizeof(b));
    fill_item(b.one, a, tiles, bf16, aggregated, wmu, 0);
    b.items = nullptr;
    b.n_items = 1;
    b.unit_tiles = 1;
    b.work = nullptr;
    b.err = err;
    b.inject_stall = inject_stall ? 1 : 0;
    b.n_kt_max = b.one.n_kt;
    b.var = a;
    // The warp-specialised kernel (the widest path tile tensor memory
    // allows): generation, MMAs and the per-row-tile epilogue overlap.  With
    // daily draws the normals bound it, and the MMA thread also issues the
    // Lhat copies (one more generator warp); with aggregated draws the MMAs
    // bound it, and a separate warp streams the copies (SPLIT).
    // RG_TC_KERNEL overrides: "simple" the phase-serial kernel (64-path
    // tiles, kept as a second implementation that the tests compare),
    // "ws64" / "ws96" cap the tile, "split" / "merged" force the copy issuer.
    const char *sel = getenv("RG_TC_KERNEL");
    const bool simple = sel && strstr(sel, "simple");
    int paths = simple ? 64 : tc_batch_paths(b.one.n_mt);
    if (sel && strstr(sel, "ws64")) paths = 64;
    if (sel && strstr(sel, "ws96") && paths > 96) paths = 96;
    bool split = aggregated;
    if (sel && strstr(sel, "split")) split = true;
    if (sel && strstr(sel, "merged")) split = false;
    b.total_tiles = (a.n_paths + paths - 1) / paths;
    b.tmem_cols = tmem_cols_for(b.one.n_mt, paths);
    if (b.one.n_mt * paths > 512) return cudaErrorInvalidValue;
    long long grid = sm_count;
    if (b.total_tiles < grid) grid = b.total_tiles;
    const bool var = a.var_mode != 0;
    if (simple)
        return var ? launch_one(mc_tc_kernel<true, false>, b, kTcThreads, tc_smem_bytes(b.n_kt_max), grid, s)
                   : launch_one(mc_tc_kernel<false, false>, b, kTcThreads, tc_smem_bytes(b.n_kt_max), grid, s);
#define RG_WS_LAUNCH(PP, SS)                                                                                      \
    return var ? launch_one(mc_tcws_kernel<true, false, PP, SS>, b, kWsThreads, WsShape<PP>::kSmem, grid, s)     \
               : launch_one(mc_tcws_kernel<false, false, PP, SS>, b, kWsThreads, WsShape<PP>::kSmem, grid, s)
    if (paths == 128) {
        if (split) RG_WS_LAUNCH(128, true);
        RG_WS_LAUNCH(128, false);
    }
    if (paths == 96) {
        if (split) RG_WS_LAUNCH(96, true);
        RG_WS_LAUNCH(96, false);
    }
    if (split) RG_WS_LAUNCH(64, true);
    RG_WS_LAUNCH(64, false);
#undef RG_WS_LAUNCH
}

// Host-side description of one batch item for tc_batch_items.
void tc_fill_batch_item(void *item_out, const PlainArgs &a, const unsigned char *tiles, int bf16,
                        bool aggregated, double wmu, long long tile_begin)
{
    fill_item(*reinterpret_cast<TcItem *>(item_out), a, tiles, bf16, aggregated, wmu, tile_begin);
}
size_t tc_item_bytes() { return sizeof(TcItem); }
long long tc_tiles_of(long long n_paths, int paths) { return (n_paths + paths - 1) / paths; }
int tc_row_tiles_of(int n) { return tc_row_tiles(n); }
int tc_k_tiles_of(int n) { return tc_k_tiles(n); }

// One persistent launch over many items: CTAs claim units of `unit_tiles`
// tiles from *work (zeroed by the caller).  The items' tiles must have been
// numbered with tc_batch_paths(n_mt_max) paths per tile.  tc_batch_prepare()
// must have run (it is not a stream operation, so it stays out of graph
// captures).
cudaError_t launch_tc_batch(const void *d_items, int n_items, long long total_tiles, int unit_tiles,
                            unsigned int *work, unsigned int *err, int n_kt_max, int n_mt_max, int grid,
                            cudaStream_t s, const long long *dyn)
{
    TcBatch b;
    memset(&b, 0, sizeof(b));
    b.dyn = dyn;
    b.items = reinterpret_cast<const TcItem *>(d_items);
    b.n_items = n_items;
    b.unit_tiles = unit_tiles < 1 ? 1 : unit_tiles;
    b.total_tiles = total_tiles;
    b.work = work;
    b.err = err;
    b.n_kt_max = n_kt_max;
    const int paths = tc_batch_paths(n_mt_max);
    b.tmem_cols = tmem_cols_for(n_mt_max, paths);
    if (n_mt_max * paths > 512 || n_kt_max > kTcMaxKt) return cudaErrorInvalidValue;
    if (paths == 128)
        mc_tcws_kernel<false, true, 128, false><<<(unsigned)grid, kWsThreads, WsShape<128>::kSmem, s>>>(b);
    else if (paths == 96)
        mc_tcws_kernel<false, true, 96, false><<<(unsigned)grid, kWsThreads, WsShape<96>::kSmem, s>>>(b);
    else
        mc_tcws_kernel<false, true, 64, false><<<(unsigned)grid, kWsThreads, WsShape<64>::kSmem, s>>>(b);
    return cudaGetLastError();
}

// Resident CTAs per SM of the batched kernel for items of at most n_mt_max
// row tiles (registers and shared memory; tensor memory is checked by the
// caller).
int tc_batch_occupancy(int n_mt_max)
{
    int per_sm = 0;
    const int paths = tc_batch_paths(n_mt_max);
    const cudaError_t e =
        paths == 128 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mc_tcws_kernel<false, true, 128, false>,
                                                                     kWsThreads, WsShape<128>::kSmem)
        : paths == 96 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mc_tcws_kernel<false, true, 96, false>,
                                                                      kWsThreads, WsShape<96>::kSmem)
                      : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, mc_tcws_kernel<false, true, 64, false>,
                                                                      kWsThreads, WsShape<64>::kSmem);
    if (e != cudaSuccess) return 1;
    return per_sm < 1 ? 1 : per_sm;
}

// Raise the batched kernels' dynamic shared-memory limit; called once
// before any launch or capture.
cudaError_t tc_batch_prepare()
{
    cudaError_t e = cudaFuncSetAttribute(mc_tcws_kernel<false, true, 128, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)WsShape<128>::kSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mc_tcws_kernel<false, true, 96, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)WsShape<96>::kSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(mc_tcws_kernel<false, true, 64, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)WsShape<64>::kSmem);
    return e;
}

} // namespace rg
