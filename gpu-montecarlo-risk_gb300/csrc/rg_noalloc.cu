// rg_simulate_noalloc: rg_simulate without any allocation.
//
// Some callers of this engine cannot call cudaMalloc (or cudaMallocAsync)
// at the point where they run a query: a host that hands the GPU a fixed
// memory budget and accounts for every byte itself, a latency-critical
// loop in which a device allocation could synchronise the device or take
// a driver lock, a plugin embedded in a framework whose caching allocator
// owns the device heap.  rg_simulate carves its per-query scratch (64-bit
// counters, the VaR candidate list and histogram) from a stream-ordered
// allocation; this entry point runs the same kernels with that scratch in
// a file-scope device array instead, and selects the VaR order statistic on
// the device, so it allocates nothing, on the device or the host.
//
// The array is kNoAllocScratchBytes (1 MiB); every GPU that loads this
// library holds it until the process exits.  Its layout: a 64-byte header
// of counters, a (kVarHistBins + 2) x 8-byte histogram, a 32-byte
// selection result, then the VaR candidate list (all remaining bytes,
// kNoAllocCandidates floats).
//
// Host code cannot pass the array's name to a kernel: on the host that
// name is a stand-in, not a device address.  The first call on each device
// (with that device current) asks the runtime for the address with
// cudaGetSymbolAddress and keeps it for that device; that first call should
// therefore come before any stream capture.  Every call clears the header
// and the histogram it uses before its kernels run, and the array keeps
// whatever the last call left in it.  Calls share the one array: calls
// whose work overlaps on the GPU (concurrent calls on different streams, or
// from different host threads) race on it and must be serialised by the
// caller.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <mutex>

#include "rg_internal.cuh"

namespace rg {

int query_check(const Portfolio *p, const rg_query *q);
int query_pass_status(const Portfolio *p, const rg_query *q, cudaStream_t s);
cudaError_t query_launch(const Portfolio *p, const rg_query *q, const PlainArgs &a, int sm_count,
                         cudaStream_t s);
PlainArgs query_args(const Portfolio *p, const rg_query *q, unsigned long long *d_counts);
double quantile_normal(double prob);

static constexpr size_t kNoAllocScratchBytes = 1u << 20;
static constexpr size_t kNoAllocHeader = 64;
static constexpr size_t kNoAllocHist = 8 * (size_t)(kVarHistBins + 2);
static constexpr size_t kNoAllocSelect = 32;
static constexpr size_t kNoAllocCandOffset = kNoAllocHeader + kNoAllocHist + kNoAllocSelect;
static constexpr unsigned int kNoAllocCandidates =
    (unsigned int)((kNoAllocScratchBytes - kNoAllocCandOffset) / sizeof(float));

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

struct NoAllocHeader {
    unsigned long long counts[2];
    unsigned long long counts2[2];
    unsigned long long tail[2];
    unsigned int cand_count;
    unsigned int pad[3];
};
static_assert(sizeof(NoAllocHeader) <= kNoAllocHeader, "header");

struct NoAllocSelect {
    float value;          // the k-th smallest candidate
    unsigned int below;   // candidates strictly smaller
    double sum_below;     // their sum
    unsigned int status;  // 0 ok
    unsigned int pad[3];
};
static_assert(sizeof(NoAllocSelect) <= kNoAllocSelect, "select");

static std::mutex g_noalloc_mu;
static unsigned char *g_noalloc_ptr[64];

// Device address of the scratch array on the current device (set up on the
// first call for that device).
static int noalloc_scratch(unsigned char **out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) {
        cudaGetLastError();
        return set_error(RG_ERR_NO_DEVICE, "no CUDA device is available");
    }
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (!g_noalloc_ptr[dev]) {
        void *ptr = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
        if (e != cudaSuccess || ptr == nullptr)
            return set_error(RG_ERR_CUDA, "cudaGetSymbolAddress of the scratch array failed: %s",
                             cudaGetErrorString(e));
        g_noalloc_ptr[dev] = (unsigned char *)ptr;
    }
    *out = g_noalloc_ptr[dev];
    return RG_OK;
}

__device__ __forceinline__ unsigned int float_key(float f)
{
    const unsigned int u = __float_as_uint(f);
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// k-th smallest of n floats (0-based k < n) by 8-bit radix selection over
// the order-preserving integer keys, one CTA; then the count and FP64 sum of
// the elements strictly below it (fixed thread order: deterministic).
__global__ void __launch_bounds__(1024) noalloc_select_kernel(const float *v, unsigned int n, unsigned int k,
                                                              NoAllocSelect *res)
{
    __shared__ unsigned int hist[256];
    __shared__ unsigned int s_prefix, s_k;
    __shared__ double red[32];
    __shared__ unsigned int redc[32];
    const int tid = threadIdx.x;
    if (tid == 0) {
        s_prefix = 0u;
        s_k = k;
    }
    for (int pass = 0; pass < 4; pass++) {
        const int shift = 24 - 8 * pass;
        const unsigned int mask = pass == 0 ? 0u : (0xffffffffu << (32 - 8 * pass));
        for (int t = tid; t < 256; t += blockDim.x) hist[t] = 0u;
        __syncthreads();
        const unsigned int prefix = s_prefix;
        for (unsigned int i = tid; i < n; i += blockDim.x) {
            const unsigned int key = float_key(v[i]);
            if ((key & mask) == prefix) atomicAdd(&hist[(key >> shift) & 0xffu], 1u);
        }
        __syncthreads();
        if (tid == 0) {
            unsigned int kk = s_k, d = 0;
            while (d < 255 && hist[d] <= kk) {
                kk -= hist[d];
                d++;
            }
            s_k = kk;
            s_prefix = prefix | (d << shift);
        }
        __syncthreads();
    }
    const unsigned int key = s_prefix;
    double sum = 0.0;
    unsigned int below = 0;
    for (unsigned int i = tid; i < n; i += blockDim.x) {
        const unsigned int ki = float_key(v[i]);
        if (ki < key) {
            sum += (double)v[i];
            below++;
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        below += __shfl_xor_sync(0xffffffffu, below, o);
    }
    if ((tid & 31) == 0) {
        red[tid >> 5] = sum;
        redc[tid >> 5] = below;
    }
    __syncthreads();
    if (tid == 0) {
        double t = 0.0;
        unsigned int c = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); w++) {
            t += red[w];
            c += redc[w];
        }
        const unsigned int u = (key & 0x80000000u) ? (key & 0x7fffffffu) : ~key;
        res->value = __uint_as_float(u);
        res->below = c;
        res->sum_below = t;
        res->status = 0u;
    }
}

} // namespace rg

using namespace rg;

#define NA_TRY(call)                                                                               \
    do {                                                                                           \
        cudaError_t e_ = (call);                                                                   \
        if (e_ != cudaSuccess)                                                                     \
            return set_error(RG_ERR_CUDA, "%s failed: %s", #call, cudaGetErrorString(e_));         \
    } while (0)

extern "C" int rg_simulate_noalloc(const rg_portfolio *h, const rg_query *q, rg_result *out, void *stream)
{
    if (!h || !out) return set_error(RG_ERR_INVALID, "NULL argument");
    const Portfolio *p = reinterpret_cast<const Portfolio *>(h);
    int st = query_check(p, q);
    if (st) return st;
    // the caller's stream, else the default stream (no stream is created)
    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms <= 0) {
        cudaGetLastError();
        return set_error(RG_ERR_NO_DEVICE, "no CUDA device is available");
    }
    const bool want_var = q->var_level > 0.0;
    const int64_t M = q->n_paths;
    const int64_t T = want_var ? rg_tail_count(M, q->var_level) : 0;

    double band_lo = 0.0, band_hi = 0.0, sd = 0.0, mean = 0.0;
    if (want_var) {
        mean = (double)q->horizon * p->wmu;
        sd = std::sqrt((double)q->horizon * p->wsw);
        const double alpha = q->var_level;
        const double z = quantile_normal(1.0 - alpha);
        const double dens = std::exp(-0.5 * z * z) / std::sqrt(2.0 * M_PI) / sd;
        const double se = std::sqrt(alpha * (1.0 - alpha) / (double)M) / dens;
        const double half = 10.0 * se + 1e-3 * sd;
        // RG_FAULT_INJECT=varband displaces the band by 5 sd, as in
        // rg_simulate (host-side injection that exercises the fallback)
        const char *inj = getenv("RG_FAULT_INJECT");
        const double shift = (inj && strstr(inj, "varband")) ? 5.0 * sd : 0.0;
        band_lo = mean + sd * z - half + shift;
        band_hi = mean + sd * z + half + shift;
        const double expect = (double)M * dens * 2.0 * half;
        if (4.0 * expect + 4096.0 > (double)kNoAllocCandidates)
            return set_error(RG_ERR_UNSUPPORTED,
                             "rg_simulate_noalloc holds at most %u VaR candidates in its %zu-byte "
                             "scratch array; this query (n_paths=%lld) needs about %.0f: use rg_simulate",
                             kNoAllocCandidates, kNoAllocScratchBytes, (long long)M, 4.0 * expect + 4096.0);
    }
    unsigned char *base = nullptr;
    st = noalloc_scratch(&base);
    if (st) return st;
    NoAllocHeader *dh = (NoAllocHeader *)base;
    unsigned long long *dhist = (unsigned long long *)(base + kNoAllocHeader);
    NoAllocSelect *dsel = (NoAllocSelect *)(base + kNoAllocHeader + kNoAllocHist);
    float *dcand = (float *)(base + kNoAllocCandOffset);

    NA_TRY(cudaMemsetAsync(dh, 0, sizeof(NoAllocHeader), s));
    PlainArgs a = query_args(p, q, dh->counts);
    if (want_var) {
        a.var_mode = 1;
        a.sel_bins = 1;
        a.sel_target = 0;
        a.sel_lo = (float)band_lo;
        a.sel_inv_w = (float)(1.0 / (band_hi - band_lo));
        a.cand = dcand;
        a.cand_count = &dh->cand_count;
        a.cand_cap = kNoAllocCandidates;
        a.tail = dh->tail;
        a.hist = dhist;
    }
    NA_TRY(query_launch(p, q, a, sms, s));
    NoAllocHeader hh;
    NA_TRY(cudaMemcpyAsync(&hh, dh, sizeof(hh), cudaMemcpyDeviceToHost, s));
    NA_TRY(cudaStreamSynchronize(s));
    // a tensor-core pass whose bounded wait ran out left incomplete counts
    st = query_pass_status(p, q, s);
    if (st) return st;
    int passes = 1;
    int64_t n_tail = (int64_t)hh.tail[0];
    if (want_var && !(n_tail < T && T <= n_tail + (int64_t)hh.cand_count && hh.cand_count <= kNoAllocCandidates)) {
        unsigned long long hist[kVarHistBins + 2];
        NA_TRY(cudaMemsetAsync(dhist, 0, sizeof(hist), s));
        a.counts = dh->counts2;
        a.var_mode = 2;
        a.sel_bins = kVarHistBins;
        a.sel_lo = (float)(mean - 12.0 * sd);
        a.sel_inv_w = (float)(kVarHistBins / (24.0 * sd));
        NA_TRY(query_launch(p, q, a, sms, s));
        NA_TRY(cudaMemcpyAsync(hist, dhist, sizeof(hist), cudaMemcpyDeviceToHost, s));
        NA_TRY(cudaStreamSynchronize(s));
        st = query_pass_status(p, q, s);
        if (st) return st;
        int64_t cum = 0;
        int j = 0;
        for (; j < kVarHistBins + 2; j++) {
            if (cum + (int64_t)hist[j] >= T) break;
            cum += (int64_t)hist[j];
        }
        if (j >= kVarHistBins + 2) return set_error(RG_ERR_CUDA, "VaR histogram holds fewer than %lld paths", (long long)T);
        if (hist[j] > kNoAllocCandidates)
            return set_error(RG_ERR_UNSUPPORTED,
                             "rg_simulate_noalloc: the VaR bin holds %llu paths, more than the %u its "
                             "scratch array can keep: use rg_simulate", hist[j], kNoAllocCandidates);
        a.var_mode = 1;
        a.sel_target = j - 1;
        NA_TRY(cudaMemsetAsync(dh->tail, 0, sizeof(dh->tail) + sizeof(dh->cand_count), s));
        NA_TRY(query_launch(p, q, a, sms, s));
        NA_TRY(cudaMemcpyAsync(&hh.tail, dh->tail, sizeof(hh.tail), cudaMemcpyDeviceToHost, s));
        NA_TRY(cudaMemcpyAsync(&hh.cand_count, &dh->cand_count, sizeof(hh.cand_count), cudaMemcpyDeviceToHost, s));
        NA_TRY(cudaStreamSynchronize(s));
        st = query_pass_status(p, q, s);
        if (st) return st;
        n_tail = (int64_t)hh.tail[0];
        passes = 3;
        if (n_tail != cum || hh.cand_count != hist[j])
            return set_error(RG_ERR_CUDA, "VaR select pass disagrees with its histogram");
    }
    memset(out, 0, sizeof(*out));
    out->n_paths = M;
    out->crash_count = (int64_t)hh.counts[0];
    out->breach_count = (int64_t)hh.counts[1];
    rg_estimator_stats(out->crash_count, M, &out->p_crash, &out->se_crash, &out->ci_lower, &out->ci_upper);
    rg_estimator_stats(out->breach_count, M, &out->p_breach, &out->se_breach, nullptr, nullptr);
    out->var = NAN;
    out->cvar = NAN;
    out->ms_device = 0.f; // not timed: no timing events are created here
    if (want_var) {
        const unsigned int kth = (unsigned int)(T - n_tail - 1);
        noalloc_select_kernel<<<1, 1024, 0, s>>>(dcand, hh.cand_count, kth, dsel);
        NA_TRY(cudaGetLastError());
        NoAllocSelect hs;
        NA_TRY(cudaMemcpyAsync(&hs, dsel, sizeof(hs), cudaMemcpyDeviceToHost, s));
        NA_TRY(cudaStreamSynchronize(s));
        // the kth+1 smallest candidates: those below the k-th value plus copies of it
        const double with_ties = hs.sum_below + (double)(kth + 1 - hs.below) * (double)hs.value;
        out->var = -(double)hs.value;
        out->cvar = ((double)(long long)hh.tail[1] * 0x1p-32 - with_ties) / (double)T;
        out->tail_count = T;
        out->var_passes = passes;
    }
    return RG_OK;
}
