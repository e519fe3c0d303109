// Batched form: many (portfolio, query) items in one persistent launch of
// the tensor-core kernel, replayed from a captured CUDA graph, with the
// work-unit size and CTA count picked by the engine's own autotuner.
//
// A batch owns: the device item table (one TcItem per query: factor tiles,
// thresholds, Philox keys, counters, first global tile), per-item 64-bit
// counters, the unit counter and error word, a pinned host copy of the
// counters, and an instantiated graph of
//     memset(counters, unit counter, error word) -> persistent kernel ->
//     copy counters and error word to pinned host memory.
// rg_batch_launch replays the graph on a stream; rg_batch_wait waits for it
// and turns the counts into estimates.
//
// Autotuner: for a batch's shape class (K tiles of the largest item, total
// 64-path tiles rounded to a power of two) it times every candidate
// (tiles per work unit in {1, 2, 4, 8, 16}) x (CTAs per SM in {1, 2} where
// shared and tensor memory allow) with CUDA events and keeps the fastest in
// a JSON file (RG_TUNE_CACHE, default ./riskgpu_tune.json), which later
// batches of the same class read.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "rg_internal.cuh"

namespace rg {

int query_check(const Portfolio *p, const rg_query *q);
PlainArgs query_args(const Portfolio *p, const rg_query *q, unsigned long long *d_counts);

struct Batch {
    int count = 0;
    int device = 0;
    int sm_count = 0;
    long long total_tiles = 0;
    int n_kt_max = 0, n_mt_max = 0;
    int unit_tiles = 2;
    int ctas_per_sm = 1;
    bool use_graph = true;
    bool tuned = false;
    unsigned char *d_items = nullptr;
    unsigned long long *d_counts = nullptr; // [count][2]
    unsigned int *d_work = nullptr;         // [0] unit counter, [1] error word
    unsigned long long *h_counts = nullptr; // pinned [count][2]
    unsigned int *h_err = nullptr;          // pinned [1]
    std::vector<rg_query> queries;
    cudaStream_t cap_stream = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    float last_ms = 0.f;
};

// ---------------------------------------------------------------- tuner cache
static std::mutex g_tune_mu;

static std::string tune_path()
{
    const char *e = getenv("RG_TUNE_CACHE");
    return (e && e[0]) ? std::string(e) : std::string("riskgpu_tune.json");
}

static std::string tune_key(const Batch *b)
{
    long long t = 1;
    while (t < b->total_tiles) t <<= 1;
    char k[96];
    snprintf(k, sizeof k, "tc_batch:nkt=%d:nmt=%d:tiles=%lld:sms=%d", b->n_kt_max, b->n_mt_max, t, b->sm_count);
    return std::string(k);
}

// The cache is a flat JSON object {"key": [unit_tiles, ctas_per_sm, ms], ...}.
static std::map<std::string, std::vector<double>> tune_load()
{
    std::map<std::string, std::vector<double>> m;
    FILE *f = fopen(tune_path().c_str(), "r");
    if (!f) return m;
    std::string s;
    char buf[4096];
    size_t got;
    while ((got = fread(buf, 1, sizeof buf, f)) > 0) s.append(buf, got);
    fclose(f);
    size_t pos = 0;
    while ((pos = s.find('"', pos)) != std::string::npos) {
        const size_t end = s.find('"', pos + 1);
        if (end == std::string::npos) break;
        const std::string key = s.substr(pos + 1, end - pos - 1);
        const size_t lb = s.find('[', end), rb = s.find(']', end);
        if (lb == std::string::npos || rb == std::string::npos || rb < lb) break;
        std::vector<double> v;
        const std::string body = s.substr(lb + 1, rb - lb - 1);
        const char *c = body.c_str();
        while (*c) {
            char *next = nullptr;
            const double x = strtod(c, &next);
            if (next == c) break;
            v.push_back(x);
            c = next;
            while (*c == ',' || *c == ' ') c++;
        }
        m[key] = v;
        pos = rb + 1;
    }
    return m;
}

static void tune_store(const std::map<std::string, std::vector<double>> &m)
{
    const std::string path = tune_path(), tmp = path + ".tmp";
    FILE *f = fopen(tmp.c_str(), "w");
    if (!f) return;
    fprintf(f, "{\n");
    size_t i = 0;
    for (const auto &kv : m) {
        fprintf(f, "  \"%s\": [", kv.first.c_str());
        for (size_t j = 0; j < kv.second.size(); j++) fprintf(f, "%s%.6g", j ? ", " : "", kv.second[j]);
        fprintf(f, "]%s\n", ++i < m.size() ? "," : "");
    }
    fprintf(f, "}\n");
    fclose(f);
    rename(tmp.c_str(), path.c_str());
}

// ---------------------------------------------------------------- helpers
static cudaError_t enqueue(Batch *b, cudaStream_t s)
{
    cudaError_t e = cudaMemsetAsync(b->d_counts, 0, sizeof(unsigned long long) * 2 * (size_t)b->count, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->d_work, 0, 2 * sizeof(unsigned int), s);
    if (e == cudaSuccess)
        e = launch_tc_batch(b->d_items, b->count, b->total_tiles, b->unit_tiles, b->d_work, b->d_work + 1,
                            b->n_kt_max, b->n_mt_max, b->sm_count * b->ctas_per_sm, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->h_counts, b->d_counts, sizeof(unsigned long long) * 2 * (size_t)b->count,
                            cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(b->h_err, b->d_work + 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, s);
    return e;
}

static int capture(Batch *b)
{
    if (b->exec) {
        cudaGraphExecDestroy(b->exec);
        b->exec = nullptr;
    }
    if (!b->use_graph) return RG_OK;
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamBeginCapture(b->cap_stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const cudaError_t e2 = enqueue(b, b->cap_stream);
        e = cudaStreamEndCapture(b->cap_stream, &g);
        if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_error(RG_ERR_CUDA, "batch graph capture failed: %s", cudaGetErrorString(e));
    return RG_OK;
}

// CTAs per SM the kernel's registers, shared and tensor memory allow.
static int max_ctas_per_sm(const Batch *b)
{
    int cols = 32;
    while (cols < b->n_mt_max * tc_batch_paths(b->n_mt_max)) cols <<= 1;
    const int by_tmem = 512 / cols, by_occ = tc_batch_occupancy(b->n_mt_max);
    int c = by_occ < by_tmem ? by_occ : by_tmem;
    return c < 1 ? 1 : (c > 2 ? 2 : c);
}

static void destroy_batch(Batch *b)
{
    if (!b) return;
    if (b->exec) cudaGraphExecDestroy(b->exec);
    if (b->cap_stream) cudaStreamDestroy(b->cap_stream);
    if (b->ev0) cudaEventDestroy(b->ev0);
    if (b->ev1) cudaEventDestroy(b->ev1);
    cudaFree(b->d_items);
    cudaFree(b->d_counts);
    cudaFree(b->d_work);
    cudaFreeHost(b->h_counts);
    cudaFreeHost(b->h_err);
    delete b;
}

} // namespace rg

using namespace rg;

extern "C" {

int rg_batch_create(const rg_batch_item *items, int32_t count, int32_t flags, rg_batch **out)
{
    if (!out) return set_error(RG_ERR_INVALID, "out is NULL");
    *out = nullptr;
    if (!items || count < 1) return set_error(RG_ERR_INVALID, "a batch needs at least one item");
    for (int i = 0; i < count; i++) {
        const Portfolio *p = reinterpret_cast<const Portfolio *>(items[i].portfolio);
        if (!p) return set_error(RG_ERR_INVALID, "batch item %d has no portfolio", i);
        int st = query_check(p, &items[i].query);
        if (st) return st;
        const rg_query &q = items[i].query;
        if (q.rng != RG_RNG_PHILOX) return set_error(RG_ERR_UNSUPPORTED, "batch item %d: batches use the Philox layout", i);
        if (q.var_level > 0.0) return set_error(RG_ERR_UNSUPPORTED, "batch item %d: VaR/CVaR are per query (rg_simulate)", i);
        if (p->n > tc_max_n() || !p->d_tc[0])
            return set_error(RG_ERR_UNSUPPORTED, "batch item %d: N = %d exceeds the batched form's limit %d", i, p->n, tc_max_n());
    }
    Batch *b = new Batch();
    b->count = count;
    b->use_graph = !(flags & RG_BATCH_NO_GRAPH);
    int st = RG_OK;
    std::vector<unsigned char> host((size_t)count * tc_item_bytes());
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sm_count, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_items, host.size());
    if (e == cudaSuccess) e = cudaMalloc(&b->d_counts, sizeof(unsigned long long) * 2 * (size_t)count);
    if (e == cudaSuccess) e = cudaMalloc(&b->d_work, 2 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_counts, sizeof(unsigned long long) * 2 * (size_t)count);
    if (e == cudaSuccess) e = cudaMallocHost(&b->h_err, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->cap_stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&b->ev1);
    if (e == cudaSuccess) e = tc_batch_prepare();
    if (e != cudaSuccess) {
        destroy_batch(b);
        return set_error(e == cudaErrorMemoryAllocation ? RG_ERR_NOMEM : RG_ERR_CUDA, "batch setup failed: %s",
                         cudaGetErrorString(e));
    }
    // the tile width follows the largest item (tensor-memory columns)
    for (int i = 0; i < count; i++) {
        const Portfolio *p = reinterpret_cast<const Portfolio *>(items[i].portfolio);
        const int kt = tc_k_tiles_of(p->n), mt = tc_row_tiles_of(p->n);
        if (kt > b->n_kt_max) b->n_kt_max = kt;
        if (mt > b->n_mt_max) b->n_mt_max = mt;
    }
    const int paths = tc_batch_paths(b->n_mt_max);
    long long tile = 0;
    for (int i = 0; i < count; i++) {
        const Portfolio *p = reinterpret_cast<const Portfolio *>(items[i].portfolio);
        const rg_query &q = items[i].query;
        const int bf16 = q.precision == RG_PREC_BF16X3 ? 1 : 0;
        PlainArgs a = query_args(p, &q, b->d_counts + 2 * (size_t)i);
        tc_fill_batch_item(host.data() + (size_t)i * tc_item_bytes(), a, p->d_tc[bf16], bf16,
                           q.draw_mode == RG_DRAWS_AGGREGATED, p->wmu, tile);
        tile += tc_tiles_of(q.n_paths, paths);
        b->queries.push_back(q);
    }
    b->total_tiles = tile;
    e = cudaMemcpy(b->d_items, host.data(), host.size(), cudaMemcpyHostToDevice);
    if (e != cudaSuccess) {
        destroy_batch(b);
        return set_error(RG_ERR_CUDA, "batch upload failed: %s", cudaGetErrorString(e));
    }
    // tuned parameters for this shape class, if any
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        const auto m = tune_load();
        const auto it = m.find(tune_key(b));
        if (it != m.end() && it->second.size() >= 2) {
            b->unit_tiles = (int)it->second[0];
            b->ctas_per_sm = (int)it->second[1];
            if (b->ctas_per_sm > max_ctas_per_sm(b)) b->ctas_per_sm = 1;
            b->tuned = true;
        }
    }
    if (!b->tuned) {
        // default: about 16 units per CTA for balance, at least one tile each
        long long u = b->total_tiles / ((long long)b->sm_count * 16);
        b->unit_tiles = (int)(u < 1 ? 1 : (u > 16 ? 16 : u));
    }
    st = capture(b);
    if (st) {
        destroy_batch(b);
        return st;
    }
    *out = reinterpret_cast<rg_batch *>(b);
    return RG_OK;
}

int rg_batch_launch(rg_batch *h, void *stream)
{
    if (!h) return set_error(RG_ERR_INVALID, "batch is NULL");
    Batch *b = reinterpret_cast<Batch *>(h);
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaEventRecord(b->ev0, s);
    if (e == cudaSuccess) e = b->exec ? cudaGraphLaunch(b->exec, s) : enqueue(b, s);
    if (e == cudaSuccess) e = cudaEventRecord(b->ev1, s);
    if (e != cudaSuccess) return set_error(RG_ERR_CUDA, "batch launch failed: %s", cudaGetErrorString(e));
    return RG_OK;
}

int rg_batch_wait(rg_batch *h, rg_result *results)
{
    if (!h) return set_error(RG_ERR_INVALID, "batch is NULL");
    Batch *b = reinterpret_cast<Batch *>(h);
    cudaError_t e = cudaEventSynchronize(b->ev1);
    if (e != cudaSuccess) return set_error(RG_ERR_CUDA, "batch failed: %s", cudaGetErrorString(e));
    cudaEventElapsedTime(&b->last_ms, b->ev0, b->ev1);
    if (*b->h_err) return set_error(RG_ERR_TIMEOUT, "batched kernel gave up a bounded wait (error word 0x%x)", *b->h_err);
    if (results) {
        for (int i = 0; i < b->count; i++) {
            rg_result &r = results[i];
            memset(&r, 0, sizeof(r));
            const int64_t M = b->queries[(size_t)i].n_paths;
            r.n_paths = M;
            r.crash_count = (int64_t)b->h_counts[2 * i];
            r.breach_count = (int64_t)b->h_counts[2 * i + 1];
            rg_estimator_stats(r.crash_count, M, &r.p_crash, &r.se_crash, &r.ci_lower, &r.ci_upper);
            rg_estimator_stats(r.breach_count, M, &r.p_breach, &r.se_breach, nullptr, nullptr);
            r.var = NAN;
            r.cvar = NAN;
            r.ms_device = b->last_ms;
        }
    }
    return RG_OK;
}

int rg_batch_info_get(const rg_batch *h, rg_batch_info *out)
{
    if (!h || !out) return set_error(RG_ERR_INVALID, "NULL argument");
    const Batch *b = reinterpret_cast<const Batch *>(h);
    out->items = b->count;
    out->total_tiles = b->total_tiles;
    out->unit_tiles = b->unit_tiles;
    out->ctas_per_sm = b->ctas_per_sm;
    out->grid = b->sm_count * b->ctas_per_sm;
    out->graph = b->exec ? 1 : 0;
    out->tuned = b->tuned ? 1 : 0;
    out->last_ms = b->last_ms;
    return RG_OK;
}

int rg_batch_tune(rg_batch *h, void *stream)
{
    if (!h) return set_error(RG_ERR_INVALID, "batch is NULL");
    Batch *b = reinterpret_cast<Batch *>(h);
    cudaStream_t s = (cudaStream_t)stream;
    const int units[] = {1, 2, 4, 8, 16};
    const int maxc = max_ctas_per_sm(b);
    float best = 1e30f;
    int best_u = b->unit_tiles, best_c = b->ctas_per_sm;
    const bool graph = b->use_graph;
    b->use_graph = false;
    for (int c = 1; c <= maxc; c++) {
        for (int u : units) {
            b->unit_tiles = u;
            b->ctas_per_sm = c;
            float ms = 0.f;
            cudaError_t e = enqueue(b, s); // warm-up
            if (e == cudaSuccess) e = cudaEventRecord(b->ev0, s);
            if (e == cudaSuccess) e = enqueue(b, s);
            if (e == cudaSuccess) e = cudaEventRecord(b->ev1, s);
            if (e == cudaSuccess) e = cudaEventSynchronize(b->ev1);
            if (e != cudaSuccess) {
                b->use_graph = graph;
                return set_error(RG_ERR_CUDA, "tuning run failed: %s", cudaGetErrorString(e));
            }
            if (*b->h_err) {
                b->use_graph = graph;
                return set_error(RG_ERR_TIMEOUT, "tuning run gave up a bounded wait");
            }
            cudaEventElapsedTime(&ms, b->ev0, b->ev1);
            if (ms < best) {
                best = ms;
                best_u = u;
                best_c = c;
            }
        }
    }
    b->unit_tiles = best_u;
    b->ctas_per_sm = best_c;
    b->use_graph = graph;
    b->tuned = true;
    {
        std::lock_guard<std::mutex> lk(g_tune_mu);
        auto m = tune_load();
        m[tune_key(b)] = {(double)best_u, (double)best_c, (double)best};
        tune_store(m);
    }
    return capture(b);
}

int rg_batch_destroy(rg_batch *h)
{
    destroy_batch(reinterpret_cast<Batch *>(h));
    return RG_OK;
}

} // extern "C"
