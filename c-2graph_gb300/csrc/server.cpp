// Serving loop with continuous batching, state resident on the device.
//
// Replaces the reference's C^2graph-PM scheduler (src/sssp/purn-perk/Main.cu:87-246):
// there a host loop alternates single-query launches on two streams and ships state to
// a CPU thread.  Here:
//   * one worker thread per query kind (SSSP, PPR, adsorption), each with its own CUDA
//     stream and workspace (a view handle sharing the graph's device arrays);
//   * requests wait in a per-kind queue; whenever a kind's previous batch finishes, its
//     worker admits every waiting request the HBM budget allows, so requests that
//     arrive while others run join the next batch of their kind, and the three kinds'
//     batches run on the device at the same time (each batched launch uses a share of
//     the SMs, so the persistent kernels are co-resident);
//   * admission by HBM footprint: each kind gets a third of the budget and a batch
//     holds at most budget / (state bytes of one query) queries;
//   * latency = completion time - submit time per request; p50/p99 over all completed.
// Results are those of c2g_sssp_batch / c2g_ppr_batch / c2g_adsorption for the same
// inputs: a request's result does not depend on what it is batched with.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <mutex>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/c2graph.h"
#include "host_io.h"
#include "internal.h"

namespace c2g {
int build_reverse_graph(c2g_graph* g);
void graph_free_view(c2g_graph* g);
}  // namespace c2g

using namespace c2g;

namespace {

using Clock = std::chrono::steady_clock;

struct Pending {
    int64_t ticket;
    c2g_request req;
    std::vector<int32_t> seeds;  // adsorption seeds (copied)
    Clock::time_point t_submit;
};

struct Done {
    int status;
    double latency_ms;
};

}  // namespace

struct c2g_server {
    c2g_graph* base = nullptr;
    c2g_graph* views[3] = {nullptr, nullptr, nullptr};
    c2g_server_config cfg{};
    std::vector<float> p_inj, p_cont, p_abnd;
    int64_t bytes_per_query[3] = {0, 0, 0};
    int64_t budget_per_kind = 0;
    std::mutex mu;
    std::condition_variable cv_work, cv_done;
    std::deque<Pending> queue[3];
    std::map<int64_t, Done> done;
    std::vector<double> latencies;
    int64_t next_ticket = 1;
    int64_t batches[3] = {0, 0, 0};
    int64_t completed = 0;
    int64_t max_batch_seen = 0;
    bool stop = false;
    std::thread workers[3];
    Clock::time_point t_first_submit, t_last_done;
    bool any_submit = false;
};

namespace {

void run_batch(c2g_server* s, int kind, std::vector<Pending>& batch) {
    c2g_graph* g = s->views[kind];
    const int n = (int)batch.size();
    const size_t V = (size_t)g->V;
    std::vector<int> status(n, C2G_OK);
    std::vector<Clock::time_point> t_done(n);  // when each request's result was complete
    if (kind == C2G_REQ_SSSP) {
        std::vector<int32_t> src(n);
        for (int i = 0; i < n; ++i) src[i] = batch[i].req.source;
        std::vector<int32_t> outv((size_t)n * V);
        int32_t* out = outv.data();
        c2g_stats st;
        const int rc = c2g_sssp_batch(g, n, src.data(), 0, C2G_SEEDS_COMPAT, out, 0, C2G_LAYOUT_QUERY_MAJOR, &st);
        for (int i = 0; i < n; ++i) {
            status[i] = rc;
            if (!rc && batch[i].req.out) std::memcpy(batch[i].req.out, out + (size_t)i * V, sizeof(int32_t) * V);
        }
        std::fill(t_done.begin(), t_done.end(), Clock::now());
    } else if (kind == C2G_REQ_PPR) {
        std::vector<int32_t> src(n);
        for (int i = 0; i < n; ++i) src[i] = batch[i].req.source;
        std::vector<float> prv((size_t)n * V);
        float* pr = prv.data();
        c2g_ppr_params p;
        c2g_ppr_default_params(g, 0, &p);
        p.alpha = s->cfg.alpha;
        p.rmax = s->cfg.rmax;
        p.r0 = 1.0f;
        p.pr0 = s->cfg.alpha;
        p.seeded = 0;
        c2g_stats st;
        const int rc = c2g_ppr_batch(g, n, src.data(), &p, pr, nullptr, 0, C2G_LAYOUT_QUERY_MAJOR, &st);
        for (int i = 0; i < n; ++i) {
            status[i] = rc;
            if (!rc && batch[i].req.out) std::memcpy(batch[i].req.out, pr + (size_t)i * V, sizeof(float) * V);
        }
        std::fill(t_done.begin(), t_done.end(), Clock::now());
    } else {
        // Label propagation runs request by request: each result is published as soon as
        // it is complete, so a waiter does not wait for the rest of the batch.
        std::vector<float> Y(V * 16);
        for (int i = 0; i < n; ++i) {
            c2g_stats st;
            const int rc = c2g_adsorption(g, 16, batch[i].seeds.data(), s->p_inj.data(), s->p_cont.data(),
                                          s->p_abnd.data(), s->cfg.ads_iterations,
                                          batch[i].req.out ? static_cast<float*>(batch[i].req.out) : Y.data(), 0, &st);
            const auto ti = Clock::now();
            std::lock_guard<std::mutex> lk(s->mu);
            const double ms = std::chrono::duration<double, std::milli>(ti - batch[i].t_submit).count();
            s->done[batch[i].ticket] = Done{rc, ms};
            s->latencies.push_back(ms);
            s->completed += 1;
            s->t_last_done = ti;
            s->cv_done.notify_all();
        }
        std::lock_guard<std::mutex> lk(s->mu);
        s->batches[kind] += 1;
        s->max_batch_seen = std::max<int64_t>(s->max_batch_seen, n);
        return;
    }
    const auto t = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    for (int i = 0; i < n; ++i) {
        const double ms = std::chrono::duration<double, std::milli>(t_done[i] - batch[i].t_submit).count();
        s->done[batch[i].ticket] = Done{status[i], ms};
        s->latencies.push_back(ms);
    }
    s->completed += n;
    s->batches[kind] += 1;
    s->max_batch_seen = std::max<int64_t>(s->max_batch_seen, n);
    s->t_last_done = t;
    s->cv_done.notify_all();
}

void worker(c2g_server* s, int kind) {
    cudaSetDevice(s->base->device);
    const int64_t cap_mem = s->bytes_per_query[kind] > 0 ? s->budget_per_kind / s->bytes_per_query[kind] : 1;
    const int64_t cap = std::max<int64_t>(1, std::min<int64_t>(s->cfg.max_batch, cap_mem));
    for (;;) {
        std::vector<Pending> batch;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !s->queue[kind].empty(); });
            if (s->stop && s->queue[kind].empty()) return;
            while (!s->queue[kind].empty() && (int64_t)batch.size() < cap) {
                batch.push_back(std::move(s->queue[kind].front()));
                s->queue[kind].pop_front();
            }
        }
        run_batch(s, kind, batch);
    }
}

}  // namespace

extern "C" {

int c2g_server_create(c2g_graph* g, const float* p_inj, const float* p_cont, const float* p_abnd,
                      const c2g_server_config* cfg, c2g_server** out) {
    if (!g || !cfg || !out) return fail(C2G_ERR_ARG, "NULL argument");
    if (cfg->max_batch < 1 || cfg->max_batch > 1024) return fail(C2G_ERR_ARG, "max_batch must be in [1,1024]");
    if (!g->adj_w && !g->adj_f) return fail(C2G_ERR_UNSUPPORTED, "graph has no weights");
    *out = nullptr;
    c2g_server* s = new c2g_server();
    s->base = g;
    s->cfg = *cfg;
    const size_t V = (size_t)g->V;
    if (p_inj && p_cont) {
        s->p_inj.assign(p_inj, p_inj + V);
        s->p_cont.assign(p_cont, p_cont + V);
        if (p_abnd) s->p_abnd.assign(p_abnd, p_abnd + V);
        else s->p_abnd.assign(V, 0.f);
    }
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    int rc = C2G_OK;
    {
        std::lock_guard<std::mutex> lk(g->mu);
        if (g->adj_f) rc = ppr_pull_prepare(g);
    }
    for (int k = 0; k < 3 && !rc; ++k) {
        rc = graph_view(g, &s->views[k]);
        if (!rc) s->views[k]->grid_scale = 1.0f / 3.0f;
    }
    // Per-query device state (bytes) and the admission budget.
    const int64_t W = 1;  // words per query amortise to 1/32 per query; counted per query
    s->bytes_per_query[C2G_REQ_SSSP] = (int64_t)V * (4 + 4) + (int64_t)V * 20 * W / 32;  // dist + staging + masks/queues
    s->bytes_per_query[C2G_REQ_PPR] = (int64_t)V * (4 + 8 * 6 + 4) + (int64_t)V * 12 / 32;  // pr,res,msg,rq x2,rq pairs x2,staging,masks
    s->bytes_per_query[C2G_REQ_ADSORPTION] = (int64_t)V * 16 * 4 * 3;                     // Y, acc, host-copy stage
    size_t free_b = 0, total_b = 0;
    if (!rc && cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) rc = fail(C2G_ERR_CUDA, "cudaMemGetInfo failed");
    const int64_t budget = cfg->hbm_budget_bytes > 0 ? cfg->hbm_budget_bytes : (int64_t)(0.8 * (double)free_b);
    s->budget_per_kind = budget / 3;
    if (prev >= 0) cudaSetDevice(prev);
    if (rc) {
        for (auto* v : s->views)
            if (v) graph_free_view(v);
        delete s;
        return rc;
    }
    for (int k = 0; k < 3; ++k) s->workers[k] = std::thread(worker, s, k);
    *out = s;
    return C2G_OK;
}

int c2g_server_submit(c2g_server* s, const c2g_request* req, int64_t* ticket) {
    if (!s || !req || !ticket) return fail(C2G_ERR_ARG, "NULL argument");
    if (req->kind < 0 || req->kind > 2) return fail(C2G_ERR_ARG, "bad request kind %d", req->kind);
    const int32_t V = s->base->V;
    Pending p;
    p.req = *req;
    if (req->kind == C2G_REQ_ADSORPTION) {
        if (!req->seeds || s->p_inj.empty()) return fail(C2G_ERR_ARG, "adsorption needs seeds and p_* arrays");
        p.seeds.assign(req->seeds, req->seeds + 16);
        for (int32_t v : p.seeds)
            if (v < 0 || v >= V) return fail(C2G_ERR_RANGE, "seed %d out of range", v);
    } else if (req->source < 0 || req->source >= V) {
        return fail(C2G_ERR_RANGE, "source %d out of range [0,%d)", req->source, V);
    }
    if (req->kind == C2G_REQ_SSSP && !s->base->adj_w) return fail(C2G_ERR_UNSUPPORTED, "graph has no int weights");
    if (req->kind != C2G_REQ_SSSP && !s->base->adj_f) return fail(C2G_ERR_UNSUPPORTED, "graph has no float weights");
    {
        std::lock_guard<std::mutex> lk(s->mu);
        if (s->stop) return fail(C2G_ERR_ARG, "server is shutting down");
        p.ticket = s->next_ticket++;
        p.t_submit = Clock::now();
        if (!s->any_submit) {
            s->any_submit = true;
            s->t_first_submit = p.t_submit;
        }
        *ticket = p.ticket;
        s->queue[req->kind].push_back(std::move(p));
    }
    s->cv_work.notify_all();
    return C2G_OK;
}

int c2g_server_wait(c2g_server* s, int64_t ticket, double timeout_s, int* status, double* latency_ms) {
    if (!s) return fail(C2G_ERR_ARG, "NULL server");
    std::unique_lock<std::mutex> lk(s->mu);
    const auto deadline = Clock::now() + std::chrono::duration<double>(timeout_s > 0 ? timeout_s : 1e9);
    if (!s->cv_done.wait_until(lk, deadline, [&] { return s->done.count(ticket) > 0; }))
        return fail(C2G_ERR_TIMEOUT, "request %lld not finished in time", (long long)ticket);
    const Done d = s->done[ticket];
    s->done.erase(ticket);
    if (status) *status = d.status;
    if (latency_ms) *latency_ms = d.latency_ms;
    return C2G_OK;
}

int c2g_server_get_stats(c2g_server* s, c2g_server_stats* out) {
    if (!s || !out) return fail(C2G_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(out, 0, sizeof(*out));
    out->completed = s->completed;
    for (int k = 0; k < 3; ++k) {
        out->batches[k] = s->batches[k];
        out->pending[k] = (int64_t)s->queue[k].size();
    }
    out->max_batch = s->max_batch_seen;
    if (!s->latencies.empty()) {
        std::vector<double> l = s->latencies;
        std::sort(l.begin(), l.end());
        out->p50_ms = l[(size_t)(0.50 * (double)(l.size() - 1))];
        out->p99_ms = l[(size_t)(0.99 * (double)(l.size() - 1))];
    }
    if (s->any_submit && s->completed > 0) {
        const double span = std::chrono::duration<double>(s->t_last_done - s->t_first_submit).count();
        out->queries_per_s = span > 0 ? (double)s->completed / span : 0.0;
    }
    for (int k = 0; k < 3; ++k) out->admit_cap[k] = s->bytes_per_query[k] > 0
                                                       ? std::min<int64_t>(s->cfg.max_batch,
                                                                           s->budget_per_kind / s->bytes_per_query[k])
                                                       : 0;
    return C2G_OK;
}

int c2g_server_destroy(c2g_server* s) {
    if (!s) return C2G_OK;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    for (auto& t : s->workers)
        if (t.joinable()) t.join();
    for (auto* v : s->views)
        if (v) graph_free_view(v);
    delete s;
    return C2G_OK;
}

}  // extern "C"
