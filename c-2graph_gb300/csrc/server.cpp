// Serving loop with continuous batching, state resident on the device.
//
// Replaces the reference's C^2graph-PM scheduler (src/sssp/purn-perk/Main.cu:87-246):
// there a host loop alternates single-query launches on two streams and ships a running
// query's state to a CPU thread through a pinned ring of snapshots.  Here:
//   * one worker thread per query kind (SSSP, PPR, adsorption), each on its own CUDA
//     stream; the three kinds run on the device at the same time, each batched launch on
//     a third of the SMs so the persistent kernels are co-resident;
//   * SSSP and PPR requests run in a resident batch (c2g_session): the worker runs epochs
//     of a few rounds, and between epochs it admits waiting requests into free slots, so a
//     request that arrives while others run starts at the next epoch, not after the
//     whole batch; a request completes as soon as its own query finishes;
//   * admission by HBM footprint: each kind gets a third of the budget, and its session
//     has at most budget / (state bytes of one query) slots;
//   * preemption (preempt_rounds > 0): when requests wait and every slot is taken, the
//     running query with the most rounds (at least preempt_rounds) is evicted into a
//     device-resident snapshot and the waiting request takes its slot; evicted queries
//     resume, before new requests, as slots free up (the analogue of the reference's
//     migration of long-running queries off the GPU, without leaving the device);
//   * adsorption label propagation runs request by request (fixed iteration count);
//   * latency = completion time - submit time per request; p50/p99 over all completed.
// Results are those of c2g_sssp / c2g_ppr (base mode) / c2g_adsorption for the same
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
void session_set_grid_share(c2g_session* s, float share);
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
    c2g_session* sessions[2] = {nullptr, nullptr};  // SSSP, PPR
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
    int64_t evictions = 0;
    int64_t completed = 0;
    int64_t max_batch_seen = 0;
    bool stop = false;
    std::thread workers[3];
    Clock::time_point t_first_submit, t_last_done;
    bool any_submit = false;
};

namespace {

void publish(c2g_server* s, const Pending& p, int status) {
    const auto t = Clock::now();
    std::lock_guard<std::mutex> lk(s->mu);
    const double ms = std::chrono::duration<double, std::milli>(t - p.t_submit).count();
    s->done[p.ticket] = Done{status, ms};
    s->latencies.push_back(ms);
    s->completed += 1;
    s->t_last_done = t;
    s->cv_done.notify_all();
}

// Adsorption: request by request, each result published as soon as it is complete.
void run_adsorption(c2g_server* s, std::vector<Pending>& batch) {
    c2g_graph* g = s->views[C2G_REQ_ADSORPTION];
    std::vector<float> Y((size_t)g->V * 16);
    for (auto& p : batch) {
        c2g_stats st;
        const int rc = c2g_adsorption(g, 16, p.seeds.data(), s->p_inj.data(), s->p_cont.data(), s->p_abnd.data(),
                                      s->cfg.ads_iterations, p.req.out ? static_cast<float*>(p.req.out) : Y.data(), 0,
                                      &st);
        publish(s, p, rc);
    }
    std::lock_guard<std::mutex> lk(s->mu);
    s->batches[C2G_REQ_ADSORPTION] += 1;
    s->max_batch_seen = std::max<int64_t>(s->max_batch_seen, (int64_t)batch.size());
}

// An evicted query waiting to resume.
struct Parked {
    Pending p;
    c2g_snapshot* snap;
};

// SSSP / PPR: a resident batch run in epochs; waiting requests (evicted ones first) take
// free slots between epochs.
void session_worker(c2g_server* s, int kind) {
    c2g_session* ss = s->sessions[kind];
    int32_t cap = 1;
    {
        const int64_t cap_mem = s->bytes_per_query[kind] > 0 ? s->budget_per_kind / s->bytes_per_query[kind] : 1;
        cap = (int32_t)std::max<int64_t>(1, std::min<int64_t>(s->cfg.max_batch, cap_mem));
    }
    std::vector<Pending> slot_req((size_t)cap);
    std::vector<bool> used((size_t)cap, false);
    std::deque<Parked> parked;
    std::vector<int32_t> finished((size_t)cap);
    std::vector<float> scratch((size_t)s->base->V);
    const int rounds = s->cfg.epoch_rounds > 0 ? s->cfg.epoch_rounds : 4;
    int running = 0;
    for (;;) {
        std::vector<Pending> admit;
        {
            std::unique_lock<std::mutex> lk(s->mu);
            s->cv_work.wait(lk, [&] { return s->stop || !s->queue[kind].empty() || running > 0 || !parked.empty(); });
            if (s->stop && s->queue[kind].empty() && running == 0 && parked.empty()) return;
            int room = cap - running - (int)parked.size();
            // Preemption: requests wait, no slot is free, and a query has run long enough.
            if (room <= 0 && parked.empty() && !s->queue[kind].empty() && s->cfg.preempt_rounds > 0) {
                int victim = -1, most = s->cfg.preempt_rounds - 1;
                for (int i = 0; i < cap; ++i) {
                    int32_t st = 0, r = 0;
                    if (!used[i] || c2g_session_slot(ss, i, &st, nullptr, &r) || st != 1) continue;
                    if (r > most) {
                        most = r;
                        victim = i;
                    }
                }
                c2g_snapshot* snap = nullptr;
                if (victim >= 0 && c2g_session_evict(ss, victim, &snap) == C2G_OK) {
                    parked.push_back(Parked{std::move(slot_req[victim]), snap});
                    used[victim] = false;
                    --running;
                    ++s->evictions;
                    room = 1;
                }
            }
            for (; room > 0 && !s->queue[kind].empty(); --room) {
                admit.push_back(std::move(s->queue[kind].front()));
                s->queue[kind].pop_front();
            }
        }
        // evicted queries resume first, into slots not taken by this round's admissions
        while (!parked.empty() && running + (int)admit.size() < cap) {
            int32_t slot = -1;
            const int rr = c2g_session_resume(ss, parked.front().snap, &slot);
            if (rr) {  // cannot continue: the request fails with the code
                c2g_snapshot_free(parked.front().snap);
                publish(s, parked.front().p, rr);
                parked.pop_front();
                continue;
            }
            slot_req[slot] = std::move(parked.front().p);
            used[slot] = true;
            ++running;
            parked.pop_front();
        }
        for (size_t a = 0; a < admit.size(); ++a) {
            Pending& p = admit[a];
            int32_t slot = -1;
            const int rc = c2g_session_admit(ss, p.req.source, &slot);
            if (rc == C2G_ERR_OVERFLOW) {  // no slot after all: back to the head of the queue
                std::lock_guard<std::mutex> lk(s->mu);
                for (size_t b = admit.size(); b > a; --b) s->queue[kind].push_front(std::move(admit[b - 1]));
                break;
            }
            if (rc) {
                publish(s, p, rc);
                continue;
            }
            slot_req[slot] = std::move(p);
            used[slot] = true;
            ++running;
        }
        if (running == 0) continue;
        int32_t nf = 0;
        c2g_stats st;
        int rc = c2g_session_step(ss, rounds, finished.data(), cap, &nf, &st);
        {
            std::lock_guard<std::mutex> lk(s->mu);
            s->batches[kind] += 1;
            s->max_batch_seen = std::max<int64_t>(s->max_batch_seen, running);
        }
        if (rc) {  // the epoch failed: every running request fails with its code
            for (int i = 0; i < cap; ++i)
                if (used[i]) {
                    publish(s, slot_req[i], rc);
                    used[i] = false;
                }
            running = 0;
            continue;
        }
        for (int k = 0; k < nf; ++k) {
            const int slot = finished[k];
            Pending& p = slot_req[slot];
            void* out = p.req.out ? p.req.out : scratch.data();
            const int rr = c2g_session_read(ss, slot, out, nullptr, 0, nullptr);
            publish(s, p, rr);
            used[slot] = false;
            --running;
        }
    }
}

void worker(c2g_server* s, int kind) {
    cudaSetDevice(s->base->device);
    if (kind != C2G_REQ_ADSORPTION) {
        session_worker(s, kind);
        return;
    }
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
        run_adsorption(s, batch);
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
        // the batched SSSP's pull rounds: the views share the base's reverse CSR
        if (!rc && g->adj_w && g->sssp_cfg.batch_pull_frac >= 0.f) rc = build_reverse_int(g);
    }
    for (int k = 0; k < 3 && !rc; ++k) {
        rc = graph_view(g, &s->views[k]);
        if (!rc) s->views[k]->grid_scale = 1.0f / 3.0f;
    }
    // Per-query device state (bytes) and the admission budget.  Per (vertex, query): SSSP
    // distance 4 B plus 28 B per 32 queries (mask, two frontier entries and masks, two pull
    // lookups); PPR
    // pr 4, res 8, msg 8, two pushed residuals 16 and their float pairs 16, plus 32 B per
    // 32 queries of masks and frontier entries; adsorption 16 labels x (Y, accumulator,
    // host stage).
    s->bytes_per_query[C2G_REQ_SSSP] = (int64_t)V * 4 + (int64_t)V * 28 / 32;
    s->bytes_per_query[C2G_REQ_PPR] = (int64_t)V * 52 + (int64_t)V * 32 / 32;
    s->bytes_per_query[C2G_REQ_ADSORPTION] = (int64_t)V * 16 * 4 * 3;
    size_t free_b = 0, total_b = 0;
    if (!rc && cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) rc = fail(C2G_ERR_CUDA, "cudaMemGetInfo failed");
    const int64_t budget = cfg->hbm_budget_bytes > 0 ? cfg->hbm_budget_bytes : (int64_t)(0.8 * (double)free_b);
    s->budget_per_kind = budget / 3;
    // Resident batches of SSSP and PPR with as many slots as the budget admits.
    for (int k = 0; k < 2 && !rc; ++k) {
        if ((k == C2G_REQ_SSSP && !g->adj_w) || (k == C2G_REQ_PPR && !g->adj_f)) continue;
        const int64_t cap = std::max<int64_t>(1, std::min<int64_t>(cfg->max_batch, s->budget_per_kind /
                                                                                      s->bytes_per_query[k]));
        c2g_ppr_params prm;
        c2g_ppr_default_params(g, 0, &prm);
        prm.alpha = cfg->alpha;
        prm.rmax = cfg->rmax;
        prm.r0 = 1.0f;
        prm.pr0 = cfg->alpha;
        prm.seeded = 0;
        rc = c2g_session_create(g, k, (int32_t)cap, k == C2G_REQ_PPR ? &prm : nullptr, &s->sessions[k]);
        if (!rc) session_set_grid_share(s->sessions[k], 1.0f / 3.0f);
    }
    if (prev >= 0) cudaSetDevice(prev);
    if (rc) {
        for (auto* v : s->views)
            if (v) graph_free_view(v);
        for (auto* ss : s->sessions)
            if (ss) c2g_session_free(ss);
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
    out->evictions = s->evictions;
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
    for (auto* ss : s->sessions)
        if (ss) c2g_session_free(ss);
    delete s;
    return C2G_OK;
}

}  // extern "C"
