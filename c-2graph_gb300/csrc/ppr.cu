// Single-query forward push (PPR and the reference's adsorption variant) for sm_103a:
// one persistent cooperative launch per query.
//
// Replaces calcuatePPR (reference src/ppr/base/Main.cu:122-395, src/ppr/purn/Main.cu:
// 149-428, src/adsorption/w-base/Main.cu:124-395) with the same BSP semantics:
//   round: every frontier vertex u pushes (1-alpha)*r_u*w(u,v) into msg[v];
//   then every vertex v that got a message: res[v] += msg[v]; msg[v] = 0;
//        if res[v] > rmax: pr[v] += alpha*res[v] and v joins the next frontier.
// The residual a frontier vertex pushes is captured when it is activated (it cannot
// change before its pop), so the pop (src/ppr/purn/Main.cu:251-253) needs no second
// read of res.  Phase A pushes over edge tiles exactly as the SSSP kernel does; it
// records each vertex's first message of the round in a touched list, so phase B
// visits only those vertices instead of sweeping all V (src/ppr/purn/Main.cu:379-407).
// Activated vertices without out-edges join no edge tile; they sit in a side list
// whose residual is cleared at the start of the next round, which is when the
// reference pops them (and, when the round cap ends the run first, they keep it).
#include <climits>

#include "device_common.cuh"
#include "internal.h"

namespace c2g {

struct PprParams {
    const int* row;
    const int2* adj;  // (target, float weight bits)
    unsigned E;
    int V;
    float* pr;
    float* res;
    float* msg;
    int* stamp;
    int2* q[2];
    float* qval[2];
    int* mark[2];
    int* touched;
    int* dangle;
    TraversalCtl* ctl;
    StampState* st;
    int source;
    float alpha, rmax, r0, pr0;
    float absorb;         // pr += absorb * r at activation (alpha for PPR, 1 for the adjoint)
    int n_src;            // base init over a list of distinct sources (adjoint targets)
    const int* src_list;  // nullptr: the single `source`
    const float* src_r0;
    int max_iter;
    int seeded;
    const int* seed_v;  // pruned records of the source (seeded mode)
    const float* seed_w;
    int n_rec;
    int log_tile;
    unsigned mark_cap;
    unsigned long long barrier_ns;
};

__device__ __forceinline__ FrontierOut ppr_out(const PprParams& p, int buf, int slot) {
    FrontierOut o;
    o.q = p.q[buf];
    o.val = p.qval[buf];
    o.mark = p.mark[buf];
    o.ctr = &p.ctl->qctr[slot];
    o.cap = (unsigned)p.V;
    o.mark_cap = p.mark_cap;
    o.log_tile = p.log_tile;
    o.flags = &p.ctl->flags;
    return o;
}

constexpr int kPprUnroll = 4;  // edges in flight per lane

// Phase A: push messages along the frontier's edges.  The first message a vertex gets
// in a round is the one whose atomicAdd returns 0 (msg[v] is 0 between rounds and every
// message is positive), so no separate touched flag is needed.  Messages below
// FLT_MIN are dropped: they cannot change any residual in float, and a vertex outside
// the frontier never holds a residual above rmax, so a zero message cannot activate it.
__device__ __forceinline__ void ppr_push(const PprParams& p, int buf, int slot, unsigned F, unsigned T,
                                         WarpStage& tst) {
    constexpr int U = kPprUnroll;
    const float one_m_a = 1.0f - p.alpha;
    const float* qv = p.qval[buf];
    walk_frontier_edges<U>(
        p.q[buf], p.mark[buf], p.row, F, T, p.log_tile, p.mark_cap, (unsigned)p.V, p.E, &p.ctl->flags,
        // (1-alpha)*r_u, src/ppr/purn/Main.cu:288
        [&](int, unsigned j) { return __float_as_int(one_m_a * ldcg(qv + j)); },
        [&](const bool* ok, const unsigned* idx, const int* qu) {
            int c[U];
            float m[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int2 ew = ok[u] ? __ldg(p.adj + idx[u]) : make_int2(0, 0);
                c[u] = ew.x;
                m[u] = __int_as_float(qu[u]) * __int_as_float(ew.y);
            }
            float old[U];
#pragma unroll
            for (int u = 0; u < U; ++u) old[u] = (ok[u] && m[u] >= 1.17549435e-38f) ? atomicAdd(p.msg + c[u], m[u]) : 1.0f;
#pragma unroll
            for (int u = 0; u < U; ++u)
                list_stage_push(tst, p.touched, &p.ctl->listctr[slot], (unsigned)p.V, &p.ctl->flags,
                                old[u] == 0.0f, c[u]);
        });
    list_stage_flush(tst, p.touched, &p.ctl->listctr[slot], (unsigned)p.V, &p.ctl->flags);
}

__global__ void __launch_bounds__(512, 2) ppr_persistent(const PprParams p) {
    TraversalCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned gwarp = gtid >> 5, nwarps = nthreads >> 5;
    const unsigned V = (unsigned)p.V;
    const float a = p.alpha, one_m_a = 1.0f - p.alpha;
    __shared__ StageSmem sm;
    const int wib = threadIdx.x >> 5;
    WarpStage fst{sm.v0[wib], sm.d0[wib], sm.x0[wib], 0};
    WarpStage tst{sm.v1[wib], nullptr, nullptr, 0};

    int sbase = p.st->stamp_base;
    const bool reset = sbase > (1 << 29);
    if (reset) sbase = 0;

    // Init: pr = res = msg = 0 (src/ppr/purn/Main.cu:156-169).
    for (unsigned v = gtid; v < V; v += nthreads) {
        p.pr[v] = 0.f;
        p.res[v] = 0.f;
        p.msg[v] = 0.f;
        if (reset) p.stamp[v] = -1;
    }
    if (!grid_sync(bar, flags, p.barrier_ns)) return;

    const int s = p.source;
    const int s_deg = __ldg(p.row + s + 1) - __ldg(p.row + s);
    if (p.src_list) {
        // Several sources with their own residual (the adjoint's target set).
        const FrontierOut out = ppr_out(p, 1, 1);
        if (gtid == 0) ctl->seeds = p.n_src;
        for (unsigned b = gwarp * 32; b < (unsigned)p.n_src; b += nwarps * 32) {
            const unsigned i = b + (unsigned)lane;
            bool want = false, dang = false;
            int v = 0, deg = 0;
            float r = 0.f;
            if (i < (unsigned)p.n_src) {
                v = p.src_list[i];
                r = p.src_r0[i];
                p.pr[v] = p.absorb * r;
                deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
                want = deg > 0;
                dang = !want;
                if (dang) p.res[v] = r;
            }
            stage_push(fst, out, want, v, deg, r);
            list_push(p.dangle, &ctl->dctr[1], (unsigned)p.V, flags, dang, v);
        }
        stage_flush(fst, out);
    } else if (!p.seeded) {
        // Base init (src/ppr/base/Main.cu:146-150): residual r0 on the source, pr0 added
        // to pr[source]; the source is the round-1 frontier and is popped (res = 0).
        if (gwarp == 0) {
            if (lane == 0) {
                p.pr[s] = p.pr0;
                ctl->seeds = 0;
                if (s_deg == 0) {
                    p.res[s] = p.r0;
                    p.dangle[0] = s;
                    ctl->dctr[1] = 1;
                }
            }
            frontier_push(ppr_out(p, 1, 1), lane == 0 && s_deg > 0, s, s_deg, p.r0);
        }
    } else {
        // Pruned-graph init (src/ppr/purn/Main.cu:78-101,173-198): pr[s] = alpha; every
        // seed, i.e. the source's pruned records followed by its kept out-edges, adds
        // (1-alpha)*alpha*w to pr and (1-alpha)*w to res; all seeds form round 1.
        const unsigned n = (unsigned)p.n_rec + (unsigned)s_deg;
        if (gtid == 0) {
            atomicAdd(p.pr + s, a);
            ctl->seeds = n;
        }
        const int rs = __ldg(p.row + s);
        for (unsigned i = gtid; i < n; i += nthreads) {
            int v;
            float w;
            if (i < (unsigned)p.n_rec) {
                v = p.seed_v[i];
                w = p.seed_w[i];
            } else {
                const int2 ew = __ldg(p.adj + rs + (int)(i - (unsigned)p.n_rec));
                v = ew.x;
                w = __int_as_float(ew.y);
            }
            atomicAdd(p.pr + v, (one_m_a * a) * w);
            atomicAdd(p.res + v, one_m_a * w);
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        const FrontierOut out = ppr_out(p, 1, 1);
        const int tag = sbase;  // distinct from every round's touched tag
        for (unsigned b = gwarp * 32; b < n; b += nwarps * 32) {
            const unsigned i = b + (unsigned)lane;
            bool want = false, dang = false;
            int v = 0, deg = 0;
            float r = 0.f;
            if (i < n) {
                v = (i < (unsigned)p.n_rec) ? p.seed_v[i] : __ldg(p.adj + rs + (int)(i - (unsigned)p.n_rec)).x;
                if (ldcg(p.stamp + v) != tag && atomicExch(p.stamp + v, tag) != tag) {
                    r = ldcg(p.res + v);
                    deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
                    want = deg > 0;
                    if (want) p.res[v] = 0.f;
                    else dang = true;
                }
            }
            stage_push(fst, out, want, v, deg, r);
            list_push(p.dangle, &ctl->dctr[1], (unsigned)p.V, flags, dang, v);
        }
        stage_flush(fst, out);
    }
    if (!grid_sync(bar, flags, p.barrier_ns)) return;

    int cur = 1, iters = 0;
    for (;;) {
        const unsigned long long c = ldcg(&ctl->qctr[cur % 3]);
        const unsigned F = (unsigned)(c >> 32), T = (unsigned)c;
        const unsigned D = ldcg(&ctl->dctr[cur % 3]);
        if (F == 0 && D == 0) break;
        if (++iters > p.max_iter) {
            // Round cap (src/ppr/purn/Main.cu:224): the activated vertices keep their
            // residual, as in the reference where they are never popped.
            if (gtid == 0) atomicOr(flags, C2G_FLAG_ITER_CAP);
            const int2* q = p.q[cur & 1];
            const float* qv = p.qval[cur & 1];
            for (unsigned j = gtid; j < F; j += nthreads) p.res[ldcg(q + j).x] = ldcg(qv + j);
            break;
        }
        // Pop the activated vertices without out-edges: their residual is dropped.
        for (unsigned j = gtid; j < D; j += nthreads) p.res[ldcg(p.dangle + j)] = 0.f;
        if (F == 0) {
            if (gtid == 0) ctl->popped += D;
            break;
        }
        const int slot = cur % 3, nslot = (cur + 1) % 3, fslot = (cur + 2) % 3;
        if (gtid == 0) {
            ctl->qctr[fslot] = 0ull;
            ctl->tilectr[fslot] = 0u;
            ctl->listctr[fslot] = 0u;
            ctl->dctr[fslot] = 0u;
            ctl->popped += F + D;
            ctl->relaxed += T;
        }
        ppr_push(p, cur & 1, slot, F, T, tst);
        if (!grid_sync(bar, flags, p.barrier_ns)) return;

        // Phase B: apply messages and activate (src/ppr/purn/Main.cu:383-391).
        const unsigned n = ldcg(&ctl->listctr[slot]);
        if (gtid == 0) ctl->touched += n;
        const FrontierOut out = ppr_out(p, (cur + 1) & 1, nslot);
        for (unsigned b = gwarp * 32; b < n; b += nwarps * 32) {
            const unsigned i = b + (unsigned)lane;
            bool want = false, dang = false;
            int v = 0, deg = 0;
            float r = 0.f;
            if (i < n) {
                v = ldcg(p.touched + i);
                r = ldcg(p.res + v) + ldcg(p.msg + v);
                p.msg[v] = 0.f;
                if (r > p.rmax) {
                    p.pr[v] = ldcg(p.pr + v) + p.absorb * r;
                    deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
                    want = deg > 0;
                    dang = !want;
                    p.res[v] = want ? 0.f : r;
                } else {
                    p.res[v] = r;
                }
            }
            stage_push(fst, out, want, v, deg, r);
            list_push(p.dangle, &ctl->dctr[nslot], (unsigned)p.V, flags, dang, v);
        }
        stage_flush(fst, out);
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        ++cur;
    }
    if (gtid == 0) {
        ctl->iterations = iters;
        p.st->stamp_base = sbase + cur + 2;
    }
}

// ---------------------------------------------------------------------------------------
// host side

static int ppr_geometry(c2g_graph* g) {
    if (g->geom_ppr.blocks > 0) return C2G_OK;
    int coop = 0;
    C2G_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device));
    if (!coop) return fail(C2G_ERR_UNSUPPORTED, "device %d lacks cooperative launch", g->device);
    int per_sm = 0;
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ppr_persistent, 512, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "PPR kernel cannot be resident (occupancy 0)");
    g->geom_ppr.blocks = per_sm * g->num_sms;
    g->geom_ppr.threads = 512;
    return C2G_OK;
}

void ppr_free(c2g_graph* g) {
    PprWork& w = g->ppr;
    void* ptrs[] = {w.pr, w.res, w.msg, w.stamp, w.q[0], w.q[1], w.qval[0], w.qval[1],
                    w.mark[0], w.mark[1], w.touched, w.dangle, w.ctl, w.st};
    for (void* ptr : ptrs)
        if (ptr) cudaFree(ptr);
    w = PprWork();
}

static int ppr_alloc(c2g_graph* g) {
    PprWork& w = g->ppr;
    const int log_tile = g->ppr_cfg.log_tile;
    if (w.msg && w.log_tile == log_tile) return C2G_OK;
    if (w.msg) ppr_free(g);
    const size_t nv = g->V ? (size_t)g->V : 1;
    const unsigned mark_cap = (unsigned)(((size_t)g->E >> log_tile) + 2);
    C2G_CUDA(cudaMalloc(&w.pr, sizeof(float) * nv));
    C2G_CUDA(cudaMalloc(&w.res, sizeof(float) * nv));
    C2G_CUDA(cudaMalloc(&w.msg, sizeof(float) * nv));
    C2G_CUDA(cudaMalloc(&w.stamp, sizeof(int) * nv));
    C2G_CUDA(cudaMalloc(&w.touched, sizeof(int) * nv));
    C2G_CUDA(cudaMalloc(&w.dangle, sizeof(int) * nv));
    for (int b = 0; b < 2; ++b) {
        C2G_CUDA(cudaMalloc(&w.q[b], sizeof(int2) * nv));
        C2G_CUDA(cudaMalloc(&w.qval[b], sizeof(float) * nv));
        C2G_CUDA(cudaMalloc(&w.mark[b], sizeof(int) * mark_cap));
    }
    C2G_CUDA(cudaMalloc(&w.ctl, sizeof(TraversalCtl)));
    C2G_CUDA(cudaMalloc(&w.st, sizeof(StampState)));
    C2G_CUDA(cudaMemsetAsync(w.stamp, 0xff, sizeof(int) * nv, g->stream));
    C2G_CUDA(cudaMemsetAsync(w.st, 0, sizeof(StampState), g->stream));
    w.mark_cap = mark_cap;
    w.log_tile = log_tile;
    return C2G_OK;
}

int ppr_launch_view(c2g_graph* g, const int32_t* row, const int2* adj, int32_t source, const c2g_ppr_params& pp,
                    float absorb, int32_t n_src, const int32_t* src_list, const float* src_r0, const int32_t* seed_v,
                    const float* seed_w, int32_t n_rec, float* pr_dev, float* res_dev, float* ms) {
    int rc;
    if ((rc = ppr_geometry(g))) return rc;
    if ((rc = ppr_alloc(g))) return rc;
    if (!adj) return fail(C2G_ERR_UNSUPPORTED, "graph has no float weights (flist / ppr wlist)");
    PprWork& w = g->ppr;
    PprParams p;
    p.row = row;
    p.adj = adj;
    p.V = g->V;
    p.E = (unsigned)g->E;
    p.pr = pr_dev ? pr_dev : w.pr;
    p.res = res_dev ? res_dev : w.res;
    p.msg = w.msg;
    p.stamp = w.stamp;
    for (int b = 0; b < 2; ++b) {
        p.q[b] = w.q[b];
        p.qval[b] = w.qval[b];
        p.mark[b] = w.mark[b];
    }
    p.touched = w.touched;
    p.dangle = w.dangle;
    p.ctl = w.ctl;
    p.st = w.st;
    p.source = source;
    p.alpha = pp.alpha;
    p.rmax = pp.rmax;
    p.r0 = pp.r0;
    p.pr0 = pp.pr0;
    p.absorb = absorb;
    p.n_src = n_src;
    p.src_list = src_list;
    p.src_r0 = src_r0;
    p.max_iter = pp.max_iter;
    p.seeded = pp.seeded;
    p.seed_v = seed_v;
    p.seed_w = seed_w;
    p.n_rec = n_rec;
    p.log_tile = w.log_tile;
    p.mark_cap = w.mark_cap;
    p.barrier_ns = 2000000000ull;
    C2G_CUDA(cudaMemsetAsync(w.ctl, 0, sizeof(TraversalCtl), g->stream));
    void* args[] = {&p};
    C2G_CUDA(cudaEventRecord(g->ev0, g->stream));
    C2G_CUDA(cudaLaunchCooperativeKernel((const void*)ppr_persistent, dim3(g->geom_ppr.blocks),
                                         dim3(g->geom_ppr.threads), args, 0, g->stream));
    C2G_CUDA(cudaEventRecord(g->ev1, g->stream));
    if (ms) {
        C2G_CUDA(cudaEventSynchronize(g->ev1));
        C2G_CUDA(cudaEventElapsedTime(ms, g->ev0, g->ev1));
    }
    return C2G_OK;
}

int ppr_launch(c2g_graph* g, int32_t source, const c2g_ppr_params& pp, const int32_t* seed_v,
               const float* seed_w, int32_t n_rec, float* pr_dev, float* res_dev, float* ms) {
    return ppr_launch_view(g, g->row, g->adj_f, source, pp, pp.alpha, 0, nullptr, nullptr, seed_v, seed_w, n_rec,
                           pr_dev, res_dev, ms);
}

}  // namespace c2g
