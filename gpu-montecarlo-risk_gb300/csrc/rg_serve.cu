// Served form: a request loop with continuous batching.
//
// Clients submit (portfolio id, query) requests; portfolios are registered
// once and stay resident (their FP64 Cholesky factor, packed and
// tensor-core tiles live on the device; the counter-based generator needs
// no other state: a query's draws are keyed by (seed, path index) alone, so
// a result does not depend on which batch or slot carried it).
//
// A scheduler thread owns `slots` preallocated launch contexts, each with
// its own stream, device item table, counters and a CUDA graph captured
// once:  memset(counters) -> persistent tensor-core kernel (item count and
// tile count read from device memory) -> copy counts to pinned host memory.
// The loop:
//   1. completions: for every busy slot whose event has fired, the counts of
//      its requests become results (latency = completion - submission) and
//      waiters are woken;
//   2. admission: if a slot is free and requests are pending, the free HBM
//      reported by cudaMemGetInfo must exceed the configured headroom;
//      otherwise the requests wait (and fail with RG_ERR_ADMISSION once they
//      have waited longer than admission_timeout_ms);
//   3. launch: up to max_batch_items pending requests (FIFO) are written to
//      the slot's pinned item table, copied to the device and the slot's
//      graph is launched; earlier slots may still be running, so new work
//      overlaps the tail of the batches already on the GPU.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "rg_internal.cuh"

namespace rg {

int query_check(const Portfolio *p, const rg_query *q);
PlainArgs query_args(const Portfolio *p, const rg_query *q, unsigned long long *d_counts);

static double now_s()
{
    return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

struct Request {
    int portfolio_id = 0;
    rg_query q;
    double t_submit = 0, t_done = 0;
    int status = RG_OK;
    bool done = false;
    rg_result result;
};

struct Slot {
    cudaStream_t stream = nullptr;
    unsigned char *d_items = nullptr;
    long long *d_dyn = nullptr;
    unsigned long long *d_counts = nullptr;
    unsigned int *d_work = nullptr;
    unsigned char *h_items = nullptr;
    long long *h_dyn = nullptr;
    unsigned long long *h_counts = nullptr;
    unsigned int *h_err = nullptr;
    cudaGraphExec_t exec = nullptr;
    cudaEvent_t done_ev = nullptr;
    std::vector<uint64_t> tickets;
    bool busy = false;
};

struct Server {
    rg_server_config cfg;
    int device = 0, sm_count = 0;
    std::map<int, const Portfolio *> portfolios;
    std::deque<uint64_t> pending;
    std::unordered_map<uint64_t, Request> reqs;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::vector<Slot> slots;
    std::thread worker;
    bool stop = false;
    uint64_t next_ticket = 1;
    std::vector<double> lat_ms;
    long long paths_done = 0, batches = 0, batched_items = 0, refused = 0;
    double t_first = 0, t_last = 0;
    int fatal = RG_OK;
};

// Row tiles of the largest servable portfolio: five (N <= 639) keeps the
// slots' launches at 96-path tiles (tensor memory: 5 x 96 columns).
static constexpr int kServedMaxRowTiles = 5;

static int slot_init(Server *sv, Slot &sl)
{
    const int cap = sv->cfg.max_batch_items;
    const size_t ib = tc_item_bytes();
    cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaMalloc(&sl.d_items, ib * (size_t)cap);
    if (e == cudaSuccess) e = cudaMalloc(&sl.d_dyn, 2 * sizeof(long long));
    if (e == cudaSuccess) e = cudaMalloc(&sl.d_counts, 16 * (size_t)cap);
    if (e == cudaSuccess) e = cudaMalloc(&sl.d_work, 2 * sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_items, ib * (size_t)cap);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_dyn, 2 * sizeof(long long));
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_counts, 16 * (size_t)cap);
    if (e == cudaSuccess) e = cudaMallocHost(&sl.h_err, sizeof(unsigned int));
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&sl.done_ev, cudaEventDisableTiming);
    if (e == cudaSuccess) e = tc_batch_prepare();
    if (e != cudaSuccess) return set_error(RG_ERR_NOMEM, "server slot setup failed: %s", cudaGetErrorString(e));
    // the slot's graph: sized for the largest item class, counts read at run time
    cudaGraph_t g = nullptr;
    e = cudaStreamBeginCapture(sl.stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        cudaError_t e2 = cudaMemsetAsync(sl.d_counts, 0, 16 * (size_t)cap, sl.stream);
        if (e2 == cudaSuccess) e2 = cudaMemsetAsync(sl.d_work, 0, 2 * sizeof(unsigned int), sl.stream);
        if (e2 == cudaSuccess)
            e2 = launch_tc_batch(sl.d_items, cap, 0, 1, sl.d_work, sl.d_work + 1, tc_max_k_tiles(),
                                 kServedMaxRowTiles, sv->sm_count, sl.stream, sl.d_dyn);
        if (e2 == cudaSuccess)
            e2 = cudaMemcpyAsync(sl.h_counts, sl.d_counts, 16 * (size_t)cap, cudaMemcpyDeviceToHost, sl.stream);
        if (e2 == cudaSuccess)
            e2 = cudaMemcpyAsync(sl.h_err, sl.d_work + 1, sizeof(unsigned int), cudaMemcpyDeviceToHost, sl.stream);
        e = cudaStreamEndCapture(sl.stream, &g);
        if (e == cudaSuccess) e = e2;
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&sl.exec, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) return set_error(RG_ERR_CUDA, "server graph capture failed: %s", cudaGetErrorString(e));
    return RG_OK;
}

static void slot_free(Slot &sl)
{
    if (sl.stream) cudaStreamSynchronize(sl.stream);
    if (sl.exec) cudaGraphExecDestroy(sl.exec);
    if (sl.done_ev) cudaEventDestroy(sl.done_ev);
    if (sl.stream) cudaStreamDestroy(sl.stream);
    cudaFree(sl.d_items);
    cudaFree(sl.d_dyn);
    cudaFree(sl.d_counts);
    cudaFree(sl.d_work);
    cudaFreeHost(sl.h_items);
    cudaFreeHost(sl.h_dyn);
    cudaFreeHost(sl.h_counts);
    cudaFreeHost(sl.h_err);
}

static void finish(Server *sv, uint64_t ticket, int status, const rg_result *r, double t)
{
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return;
    Request &rq = it->second;
    rq.status = status;
    if (r) rq.result = *r;
    rq.t_done = t;
    rq.done = true;
    if (status == RG_OK) {
        sv->lat_ms.push_back(1e3 * (t - rq.t_submit));
        sv->paths_done += rq.q.n_paths;
        if (sv->t_first == 0 || rq.t_submit < sv->t_first) sv->t_first = rq.t_submit;
        if (t > sv->t_last) sv->t_last = t;
    }
}

// One pass of the scheduler (called with sv->mu held).  Returns true if it
// did anything.
static bool schedule_once(Server *sv)
{
    bool acted = false;
    const double t = now_s();
    // 1. completions
    for (Slot &sl : sv->slots) {
        if (!sl.busy) continue;
        const cudaError_t q = cudaEventQuery(sl.done_ev);
        if (q == cudaErrorNotReady) continue;
        const int st = (q != cudaSuccess) ? RG_ERR_CUDA : (*sl.h_err ? RG_ERR_TIMEOUT : RG_OK);
        for (size_t i = 0; i < sl.tickets.size(); i++) {
            auto it = sv->reqs.find(sl.tickets[i]);
            if (it == sv->reqs.end()) continue;
            rg_result r;
            memset(&r, 0, sizeof(r));
            const int64_t M = it->second.q.n_paths;
            r.n_paths = M;
            r.crash_count = (int64_t)sl.h_counts[2 * i];
            r.breach_count = (int64_t)sl.h_counts[2 * i + 1];
            rg_estimator_stats(r.crash_count, M, &r.p_crash, &r.se_crash, &r.ci_lower, &r.ci_upper);
            rg_estimator_stats(r.breach_count, M, &r.p_breach, &r.se_breach, nullptr, nullptr);
            r.var = NAN;
            r.cvar = NAN;
            finish(sv, sl.tickets[i], st, &r, t);
        }
        sv->batches++;
        sv->batched_items += (long long)sl.tickets.size();
        sl.tickets.clear();
        sl.busy = false;
        acted = true;
    }
    if (acted) sv->cv_done.notify_all();
    // 2./3. admission and launch
    while (!sv->pending.empty()) {
        Slot *free_slot = nullptr;
        for (Slot &sl : sv->slots)
            if (!sl.busy) {
                free_slot = &sl;
                break;
            }
        if (!free_slot) break;
        size_t fr = 0, tot = 0;
        const bool mem_ok = cudaMemGetInfo(&fr, &tot) == cudaSuccess && (long long)fr > sv->cfg.headroom_bytes;
        if (!mem_ok) {
            // refuse requests that have waited too long for headroom
            while (!sv->pending.empty()) {
                const uint64_t tk = sv->pending.front();
                auto it = sv->reqs.find(tk);
                if (it != sv->reqs.end() && 1e3 * (t - it->second.t_submit) < sv->cfg.admission_timeout_ms) break;
                sv->pending.pop_front();
                sv->refused++;
                finish(sv, tk, RG_ERR_ADMISSION, nullptr, t);
                acted = true;
            }
            sv->cv_done.notify_all();
            break;
        }
        Slot &sl = *free_slot;
        long long tile = 0;
        int n = 0;
        while (!sv->pending.empty() && n < sv->cfg.max_batch_items) {
            const uint64_t tk = sv->pending.front();
            sv->pending.pop_front();
            auto it = sv->reqs.find(tk);
            if (it == sv->reqs.end()) continue;
            const Request &rq = it->second;
            const Portfolio *p = sv->portfolios[rq.portfolio_id];
            const int bf16 = rq.q.precision == RG_PREC_BF16X3 ? 1 : 0;
            PlainArgs a = query_args(p, &rq.q, sl.d_counts + 2 * (size_t)n);
            tc_fill_batch_item(sl.h_items + (size_t)n * tc_item_bytes(), a, p->d_tc[bf16], bf16,
                               rq.q.draw_mode == RG_DRAWS_AGGREGATED, p->wmu, tile);
            tile += tc_tiles_of(rq.q.n_paths, tc_batch_paths(kServedMaxRowTiles));
            sl.tickets.push_back(tk);
            n++;
        }
        if (n == 0) break;
        sl.h_dyn[0] = n;
        sl.h_dyn[1] = tile;
        cudaError_t e = cudaMemcpyAsync(sl.d_items, sl.h_items, tc_item_bytes() * (size_t)n, cudaMemcpyHostToDevice,
                                        sl.stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(sl.d_dyn, sl.h_dyn, 2 * sizeof(long long), cudaMemcpyHostToDevice, sl.stream);
        if (e == cudaSuccess) e = cudaGraphLaunch(sl.exec, sl.stream);
        if (e == cudaSuccess) e = cudaEventRecord(sl.done_ev, sl.stream);
        if (e != cudaSuccess) {
            for (uint64_t tk : sl.tickets) finish(sv, tk, RG_ERR_CUDA, nullptr, t);
            sl.tickets.clear();
            sv->cv_done.notify_all();
            sv->fatal = RG_ERR_CUDA;
            break;
        }
        sl.busy = true;
        acted = true;
    }
    return acted;
}

static void worker_main(Server *sv)
{
    cudaSetDevice(sv->device);
    std::unique_lock<std::mutex> lk(sv->mu);
    while (!sv->stop) {
        const bool acted = schedule_once(sv);
        bool busy = false;
        for (const Slot &sl : sv->slots) busy = busy || sl.busy;
        if (!acted) {
            // GPU work in flight: poll again soon; idle: sleep until a submit
            if (busy || !sv->pending.empty())
                sv->cv_work.wait_for(lk, std::chrono::microseconds(sv->cfg.poll_us));
            else
                sv->cv_work.wait_for(lk, std::chrono::milliseconds(5));
        }
    }
    // drain
    for (Slot &sl : sv->slots)
        if (sl.busy) cudaEventSynchronize(sl.done_ev);
    schedule_once(sv);
}

} // namespace rg

using namespace rg;

extern "C" {

void rg_server_default_config(rg_server_config *cfg)
{
    if (!cfg) return;
    cfg->slots = 3;
    cfg->max_batch_items = 64;
    cfg->headroom_bytes = 1ll << 30;
    cfg->admission_timeout_ms = 1000.0;
    cfg->poll_us = 20;
}

int rg_server_create(const rg_server_config *cfg, rg_server **out)
{
    if (!out) return set_error(RG_ERR_INVALID, "out is NULL");
    *out = nullptr;
    rg_server_config c;
    rg_server_default_config(&c);
    if (cfg) c = *cfg;
    if (c.slots < 1 || c.slots > 16 || c.max_batch_items < 1 || c.max_batch_items > 4096 || c.poll_us < 1)
        return set_error(RG_ERR_INVALID, "invalid server configuration");
    Server *sv = new Server();
    sv->cfg = c;
    if (cudaGetDevice(&sv->device) != cudaSuccess ||
        cudaDeviceGetAttribute(&sv->sm_count, cudaDevAttrMultiProcessorCount, sv->device) != cudaSuccess) {
        cudaGetLastError();
        delete sv;
        return set_error(RG_ERR_NO_DEVICE, "no CUDA device is available");
    }
    sv->slots.resize((size_t)c.slots);
    for (Slot &sl : sv->slots) {
        const int st = slot_init(sv, sl);
        if (st) {
            for (Slot &s2 : sv->slots) slot_free(s2);
            delete sv;
            return st;
        }
    }
    sv->worker = std::thread(worker_main, sv);
    *out = reinterpret_cast<rg_server *>(sv);
    return RG_OK;
}

int rg_server_register(rg_server *h, int32_t portfolio_id, const rg_portfolio *p)
{
    if (!h || !p) return set_error(RG_ERR_INVALID, "NULL argument");
    Server *sv = reinterpret_cast<Server *>(h);
    const Portfolio *pp = reinterpret_cast<const Portfolio *>(p);
    const int max_n = kServedMaxRowTiles * 128 - 1; // row N (w^T L) shares the last row tile
    if (pp->n > max_n || tc_row_tiles_of(pp->n) > kServedMaxRowTiles || !pp->d_tc[0] || !pp->d_tc[1])
        return set_error(RG_ERR_UNSUPPORTED, "served portfolios are limited to N <= %d", max_n);
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->portfolios[portfolio_id] = pp;
    return RG_OK;
}

int rg_server_submit(rg_server *h, int32_t portfolio_id, const rg_query *q, uint64_t *ticket)
{
    if (!h || !q || !ticket) return set_error(RG_ERR_INVALID, "NULL argument");
    Server *sv = reinterpret_cast<Server *>(h);
    std::lock_guard<std::mutex> lk(sv->mu);
    auto pit = sv->portfolios.find(portfolio_id);
    if (pit == sv->portfolios.end()) return set_error(RG_ERR_INVALID, "portfolio %d is not registered", portfolio_id);
    int st = query_check(pit->second, q);
    if (st) return st;
    if (q->rng != RG_RNG_PHILOX || q->var_level > 0.0)
        return set_error(RG_ERR_UNSUPPORTED, "served queries use the Philox layout and no VaR");
    if (sv->fatal) return set_error(sv->fatal, "the server's device work failed earlier");
    Request rq;
    rq.portfolio_id = portfolio_id;
    rq.q = *q;
    rq.q.d_s_values = nullptr;
    rq.q.d_port_values = nullptr;
    rq.t_submit = now_s();
    memset(&rq.result, 0, sizeof(rq.result));
    const uint64_t tk = sv->next_ticket++;
    sv->reqs.emplace(tk, rq);
    sv->pending.push_back(tk);
    *ticket = tk;
    sv->cv_work.notify_one();
    return RG_OK;
}

int rg_server_wait(rg_server *h, uint64_t ticket, rg_result *out, double *latency_ms)
{
    if (!h) return set_error(RG_ERR_INVALID, "server is NULL");
    Server *sv = reinterpret_cast<Server *>(h);
    std::unique_lock<std::mutex> lk(sv->mu);
    auto it = sv->reqs.find(ticket);
    if (it == sv->reqs.end()) return set_error(RG_ERR_INVALID, "unknown ticket %llu", (unsigned long long)ticket);
    sv->cv_done.wait(lk, [&] { return sv->reqs[ticket].done; });
    Request rq = sv->reqs[ticket];
    sv->reqs.erase(ticket);
    if (out) *out = rq.result;
    if (latency_ms) *latency_ms = 1e3 * (rq.t_done - rq.t_submit);
    if (rq.status != RG_OK)
        return set_error(rq.status, "request %llu failed: %s", (unsigned long long)ticket, rg_status_string(rq.status));
    return RG_OK;
}

int rg_server_stats(rg_server *h, rg_server_summary *out)
{
    if (!h || !out) return set_error(RG_ERR_INVALID, "NULL argument");
    Server *sv = reinterpret_cast<Server *>(h);
    std::lock_guard<std::mutex> lk(sv->mu);
    memset(out, 0, sizeof(*out));
    out->completed = (int64_t)sv->lat_ms.size();
    out->refused = sv->refused;
    out->batches = sv->batches;
    out->mean_batch_items = sv->batches ? (double)sv->batched_items / (double)sv->batches : 0.0;
    if (!sv->lat_ms.empty()) {
        std::vector<double> v = sv->lat_ms;
        std::sort(v.begin(), v.end());
        auto pct = [&](double f) {
            const size_t i = (size_t)std::min<double>((double)(v.size() - 1), std::ceil(f * (double)v.size()) - 1.0);
            return v[i];
        };
        out->p50_ms = pct(0.50);
        out->p99_ms = pct(0.99);
        out->max_ms = v.back();
        out->paths_per_s = (sv->t_last > sv->t_first) ? (double)sv->paths_done / (sv->t_last - sv->t_first) : 0.0;
    }
    return RG_OK;
}

int rg_server_reset_stats(rg_server *h)
{
    if (!h) return set_error(RG_ERR_INVALID, "server is NULL");
    Server *sv = reinterpret_cast<Server *>(h);
    std::lock_guard<std::mutex> lk(sv->mu);
    sv->lat_ms.clear();
    sv->paths_done = sv->batches = sv->batched_items = sv->refused = 0;
    sv->t_first = sv->t_last = 0;
    return RG_OK;
}

int rg_server_destroy(rg_server *h)
{
    if (!h) return RG_OK;
    Server *sv = reinterpret_cast<Server *>(h);
    {
        std::lock_guard<std::mutex> lk(sv->mu);
        sv->stop = true;
        sv->cv_work.notify_all();
    }
    if (sv->worker.joinable()) sv->worker.join();
    for (Slot &sl : sv->slots) slot_free(sl);
    delete sv;
    return RG_OK;
}

} // extern "C"
