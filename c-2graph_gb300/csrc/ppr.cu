// Single-query forward push (PPR and the reference's adsorption variant) for sm_103a:
// one persistent cooperative launch per query.
//
// Replaces calcuatePPR (reference src/ppr/base/Main.cu:122-395, src/ppr/purn/Main.cu:
// 149-428, src/adsorption/w-base/Main.cu:124-395) with the same BSP semantics:
//   round: every frontier vertex u pushes (1-alpha)*r_u*w(u,v) into msg[v];
//   then every vertex v that got a message: res[v] += msg[v]; msg[v] = 0;
//        if res[v] > rmax: pr[v] += alpha*res[v] and v joins the next frontier.
//
// Precision: edge weights and pr are FP32; the residual state (res, msg, the residual a
// frontier vertex pushes) is FP64.  res > rmax is a threshold: FP32 residuals of vertices
// sitting at rmax land on the other side of it than FP64 ones, each such flip moves
// about rmax of mass and cascades downstream, so FP32 residual bookkeeping drifts past
// L1 1e-6 of the FP64 result as graphs grow.  With FP64 residuals the decisions match the
// FP64 push up to summation order.
//
// Two round shapes, chosen per round from the frontier's out-edge count T:
//   * push (T small): edge-tiled walk over the frontier's out-edges, FP64 atomicAdd into
//     msg; the add that returns 0 records the target in the touched list and phase B
//     visits only touched vertices (no O(V) sweep, src/ppr/purn/Main.cu:379-407);
//   * pull (T * pull_div > E): every vertex sums (1-alpha)*r_u*w(u,v) over its in-edges
//     (reverse CSR) from a dense array qd of the frontier's pushed residuals, with a
//     segmented warp reduction (a few atomics per 32 in-edges instead of one per edge),
//     then a dense apply pass over all V.  Both shapes give the same BSP round.
// The residual a frontier vertex pushes is captured when it is activated (nothing
// changes it before its pop).  Activated vertices without out-edges sit in a side list
// whose residual is cleared at the start of the next round, which is when the reference
// pops them (when the round cap ends the run first, they keep it).
#include <climits>

#include "device_common.cuh"
#include "fp64_mul.h"
#include "internal.h"

namespace c2g {

struct PprParams {
    const int* row;
    const int2* adj;  // (target, float weight bits)
    unsigned E;
    int V;
    const int* row_r;   // reverse CSR (in-edges carrying w(u,v)), or nullptr: push only
    const int2* adj_r;
    const int* mark_r;  // owner of in-edge t * 2^kPullTileLog
    int pull_div;       // pull when T * pull_div > E (0: never)
    int dense_div;      // dense push round (no touched list) when T * dense_div > E (0: never)
    float* pr;
    double* res;
    double* msg;
    double* qd;  // (1-alpha)*r of frontier vertices, 0 elsewhere (pull rounds)
    int* stamp;
    int2* q[2];
    double* qval[2];
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
    o.val = nullptr;
    o.vald = p.qval[buf];
    o.mark = p.mark[buf];
    o.ctr = &p.ctl->qctr[slot];
    o.cap = (unsigned)p.V;
    o.mark_cap = p.mark_cap;
    o.log_tile = p.log_tile;
    o.flags = &p.ctl->flags;
    return o;
}

constexpr int kPprUnroll = 8;  // edges in flight per lane
constexpr int kPprThreads = 512;  // launch shape of the persistent push
constexpr int kPprBlocksPerSm = 2;
// Round-robin tiles in push rounds (a dynamic tile queue measured no faster: 20.2 vs 20.4 ms
// per scale-22 query).
constexpr bool kPprDynTiles = false;

// Push round, phase A.  The first message a vertex gets in a round is the one whose
// atomicAdd returns 0 (msg[v] is 0 between rounds and every message is positive), so no
// separate touched flag is needed.  Zero messages are dropped: a vertex outside the
// frontier never holds a residual above rmax, so a zero message cannot activate it.
// With track = false (a dense round) the adds are fire-and-forget red.add and the
// apply pass sweeps all vertices instead of a touched list.
__device__ __forceinline__ void ppr_push(const PprParams& p, int buf, int slot, unsigned F, unsigned T,
                                         WarpStage& tst, bool track) {
    constexpr int U = kPprUnroll;
    const double one_m_a = 1.0 - (double)p.alpha;
    const double* qv = p.qval[buf];
    walk_frontier_edges<U>(
        p.q[buf], p.mark[buf], p.row, F, T, p.log_tile, p.mark_cap, (unsigned)p.V, p.E, &p.ctl->flags,
        // (1-alpha)*r_u (src/ppr/purn/Main.cu:288); the owner is popped, so it leaves qd
        [&](int v, unsigned j) {
            if (p.qd) p.qd[v] = 0.0;
            return one_m_a * ldcg(qv + j);
        },
        [&](const bool* ok, const unsigned* idx, const double* qu) {
            int c[U];
            double m[U];
            bool send[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int2 ew = ok[u] ? __ldg(p.adj + idx[u]) : make_int2(0, 0);
                c[u] = ew.x;
                // m = qu * w in FP64, on the integer pipes (fp64_mul.h); a message is sent
                // when it is positive (w > 0: qu > 0 for every activated vertex)
                const unsigned wb = (unsigned)ew.y;
                const DSplit qs = c2g_dsplit(qu[u]);
                const bool mok = c2g_mul_q_ok(qs) && c2g_mul_w_ok(wb);
                send[u] = ok[u] && ew.y > 0;
                m[u] = c2g_mul(qs, wb);
                if (__any_sync(kFull, send[u] && !mok)) {  // w subnormal: FP64 pipe
                    if (!mok) m[u] = qu[u] * (double)__int_as_float(ew.y);
                    send[u] = send[u] && (mok || m[u] > 0.0);
                }
            }
            if (!track) {
#pragma unroll
                for (int u = 0; u < U; ++u)
                    if (send[u]) atomicAdd(p.msg + c[u], m[u]);
                return;
            }
            unsigned long long old[U];
#pragma unroll
            for (int u = 0; u < U; ++u)
                old[u] = send[u] ? c2g_dbits(atomicAdd(p.msg + c[u], m[u])) : 1ull;
#pragma unroll
            for (int u = 0; u < U; ++u)
                list_stage_push(tst, p.touched, &p.ctl->listctr[slot], (unsigned)p.V, &p.ctl->flags,
                                old[u] == 0ull, c[u]);
        },
        kPprDynTiles ? &p.ctl->tilectr[slot] : nullptr);
    if (track) list_stage_flush(tst, p.touched, &p.ctl->listctr[slot], (unsigned)p.V, &p.ctl->flags);
}

// Pull round, phase A: msg[v] = sum over in-edges (u, w) of qd[u] * w.  In-edges are
// walked in tiles of 2^kPullTileLog; 32 consecutive in-edges per step, one per lane; a
// segmented scan sums each owner's lanes and the segment's last lane adds it to msg.
__device__ __forceinline__ void ppr_pull(const PprParams& p) {
    const int lane = threadIdx.x & 31;
    const unsigned gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned tw = 1u << kPullTileLog;
    const unsigned ntiles = (p.E + tw - 1) >> kPullTileLog;
    const unsigned V = (unsigned)p.V;
    for (unsigned t = gwarp; t < ntiles; t += nwarps) {
        unsigned e0 = t << kPullTileLog;
        const unsigned e1 = min(e0 + tw, p.E);
        unsigned o = (unsigned)__ldg(p.mark_r + t);
        while (e0 < e1) {
            const unsigned j = o + (unsigned)lane;
            unsigned base = 0x7fffffffu, endv = 0xffffffffu;
            if (j < V) {
                base = (unsigned)__ldg(p.row_r + j);
                endv = (unsigned)__ldg(p.row_r + j + 1);
            }
            if (o >= V || (unsigned)__shfl_sync(kFull, (int)base, 0) > e0) {
                if (lane == 0) atomicOr(&p.ctl->flags, C2G_FLAG_BOUNDS);
                break;
            }
            const unsigned seg_end = min(e1, (unsigned)__shfl_sync(kFull, endv, 31));
            if (seg_end <= e0) {  // 32 owners without in-edges: move on (o grows to V at most)
                o += 32;
                continue;
            }
            for (unsigned eb = e0; eb < seg_end; eb += 32) {
                const unsigned e = eb + (unsigned)lane;
                const bool valid = e < seg_end;
                const int k = owner_lane(base, e);  // rows without in-edges share bases: the last one owns e
                double s = 0.0;
                if (valid) {
                    const int2 ew = __ldg(p.adj_r + e);
                    s = ldcg(p.qd + ew.x) * (double)__int_as_float(ew.y);
                }
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const double ts = __shfl_up_sync(kFull, s, off);
                    const int tk = __shfl_up_sync(kFull, k, off);
                    if (lane >= off && tk == k) s += ts;
                }
                const int kn = __shfl_down_sync(kFull, k, 1);
                const bool vn = __shfl_down_sync(kFull, (int)valid, 1) != 0;
                const bool tail = valid && (lane == 31 || !vn || kn != k);
                if (tail && s != 0.0) atomicAdd(p.msg + o + (unsigned)k, s);
            }
            e0 = seg_end;
            o += 32;
        }
    }
}

__global__ void __launch_bounds__(kPprThreads, kPprBlocksPerSm) ppr_persistent(const PprParams p) {
    TraversalCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned gwarp = gtid >> 5, nwarps = nthreads >> 5;
    const unsigned V = (unsigned)p.V;
    const double a = (double)p.alpha, one_m_a = 1.0 - (double)p.alpha, absorb = (double)p.absorb;
    const unsigned long long rmax_bits = c2g_dbits((double)p.rmax);
    __shared__ StageSmemD sm;
    const int wib = threadIdx.x >> 5;
    WarpStage fst{sm.v0[wib], sm.d0[wib], nullptr, 0, sm.xd0[wib]};
    WarpStage tst{sm.v1[wib], nullptr, nullptr, 0};
    unsigned long long tph = globaltimer_ns();

    int sbase = p.st->stamp_base;
    const bool reset = sbase > (1 << 29);
    if (reset) sbase = 0;

    // Init: pr = res = msg = 0 (src/ppr/purn/Main.cu:156-169), qd = 0.
    for (unsigned v = gtid; v < V; v += nthreads) {
        p.pr[v] = 0.f;
        p.res[v] = 0.0;
        p.msg[v] = 0.0;
        if (p.qd) p.qd[v] = 0.0;
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
            double r = 0.0;
            if (i < (unsigned)p.n_src) {
                v = p.src_list[i];
                r = (double)p.src_r0[i];
                p.pr[v] = (float)(absorb * r);
                deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
                want = deg > 0;
                dang = !want;
                if (dang) p.res[v] = r;
                if (want && p.qd) p.qd[v] = one_m_a * r;
            }
            stage_push(fst, out, want, v, deg, 0.f, r);
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
                    p.res[s] = (double)p.r0;
                    p.dangle[0] = s;
                    ctl->dctr[1] = 1;
                } else if (p.qd) {
                    p.qd[s] = one_m_a * (double)p.r0;
                }
            }
            const FrontierOut out = ppr_out(p, 1, 1);
            stage_push(fst, out, lane == 0 && s_deg > 0, s, s_deg, 0.f, (double)p.r0);
            stage_flush(fst, out);
        }
    } else {
        // Pruned-graph init (src/ppr/purn/Main.cu:78-101,173-198): pr[s] = alpha; every
        // seed, i.e. the source's pruned records followed by its kept out-edges, adds
        // (1-alpha)*alpha*w to pr and (1-alpha)*w to res; all seeds form round 1.
        const unsigned n = (unsigned)p.n_rec + (unsigned)s_deg;
        if (gtid == 0) {
            atomicAdd(p.pr + s, p.alpha);
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
            atomicAdd(p.pr + v, (float)(one_m_a * a * (double)w));
            atomicAdd(p.res + v, one_m_a * (double)w);
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        const FrontierOut out = ppr_out(p, 1, 1);
        const int tag = sbase;  // distinct from every round's tag
        for (unsigned b = gwarp * 32; b < n; b += nwarps * 32) {
            const unsigned i = b + (unsigned)lane;
            bool want = false, dang = false;
            int v = 0, deg = 0;
            double r = 0.0;
            if (i < n) {
                v = (i < (unsigned)p.n_rec) ? p.seed_v[i] : __ldg(p.adj + rs + (int)(i - (unsigned)p.n_rec)).x;
                if (ldcg(p.stamp + v) != tag && atomicExch(p.stamp + v, tag) != tag) {
                    r = __ldcg(p.res + v);
                    deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
                    want = deg > 0;
                    if (want) {
                        p.res[v] = 0.0;
                        if (p.qd) p.qd[v] = one_m_a * r;
                    } else {
                        dang = true;
                    }
                }
            }
            stage_push(fst, out, want, v, deg, 0.f, r);
            list_push(p.dangle, &ctl->dctr[1], (unsigned)p.V, flags, dang, v);
        }
        stage_flush(fst, out);
    }
    if (!grid_sync(bar, flags, p.barrier_ns)) return;
    phase_mark(ctl->phase_ns, tph, 0);

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
            const double* qv = p.qval[cur & 1];
            for (unsigned j = gtid; j < F; j += nthreads) p.res[ldcg(q + j).x] = __ldcg(qv + j);
            break;
        }
        // Pop the activated vertices without out-edges: their residual is dropped.
        for (unsigned j = gtid; j < D; j += nthreads) p.res[ldcg(p.dangle + j)] = 0.0;
        if (F == 0) {
            if (gtid == 0) ctl->popped += D;
            break;
        }
        const int slot = cur % 3, nslot = (cur + 1) % 3, fslot = (cur + 2) % 3;
        const bool pull = p.row_r && p.pull_div > 0 && (unsigned long long)T * (unsigned)p.pull_div > p.E;
        const bool dense = pull || (p.dense_div > 0 && (unsigned long long)T * (unsigned)p.dense_div > p.E);
        if (gtid == 0) {
            ctl->qctr[fslot] = 0ull;
            ctl->tilectr[fslot] = 0u;
            ctl->listctr[fslot] = 0u;
            ctl->dctr[fslot] = 0u;
            ctl->popped += F + D;
            ctl->relaxed += pull ? p.E : T;
            if (pull) ctl->pad[0] += 1;  // pull rounds
        }
        const FrontierOut out = ppr_out(p, (cur + 1) & 1, nslot);
        if (pull)
            ppr_pull(p);
        else
            ppr_push(p, cur & 1, slot, F, T, tst, !dense);
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tph, 2);
        if (!dense) {
            // Phase B: apply messages and activate (src/ppr/purn/Main.cu:383-391).
            const unsigned n = ldcg(&ctl->listctr[slot]);
            if (gtid == 0) ctl->touched += n;
            for (unsigned b = gwarp * 32; b < n; b += nwarps * 32) {
                const unsigned i = b + (unsigned)lane;
                bool want = false, dang = false;
                int v = 0, deg = 0;
                double r = 0.0;
                if (i < n) {
                    v = ldcg(p.touched + i);
                    r = __ldcg(p.res + v) + __ldcg(p.msg + v);
                    p.msg[v] = 0.0;
                    if (c2g_dbits(r) > rmax_bits) {  // both non-negative
                        p.pr[v] = ldcg(p.pr + v) + (float)(absorb * r);
                        deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
                        want = deg > 0;
                        dang = !want;
                        p.res[v] = want ? 0.0 : r;
                        if (want && p.qd) p.qd[v] = one_m_a * r;
                    } else {
                        p.res[v] = r;
                    }
                }
                stage_push(fst, out, want, v, deg, 0.f, r);
                list_push(p.dangle, &ctl->dctr[nslot], (unsigned)p.V, flags, dang, v);
            }
        } else {
            // Dense apply: every vertex (an untouched one has msg 0 and res <= rmax, so
            // it is left as it is).
            if (gtid == 0) ctl->touched += V;
            for (unsigned b = gwarp * 32; b < V; b += nwarps * 32) {
                const unsigned v = b + (unsigned)lane;
                bool want = false, dang = false;
                int deg = 0;
                double r = 0.0;
                if (v < V) {
                    const double m = __ldcg(p.msg + v);
                    const double q0 = p.qd ? __ldcg(p.qd + v) : 0.0;
                    if (c2g_dbits(m) != 0ull) {  // messages are positive; msg is +0 otherwise
                        p.msg[v] = 0.0;
                        r = __ldcg(p.res + v) + m;
                        if (c2g_dbits(r) > rmax_bits) {  // both non-negative
                            p.pr[v] = ldcg(p.pr + v) + (float)(absorb * r);
                            deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
                            want = deg > 0;
                            dang = !want;
                            p.res[v] = want ? 0.0 : r;
                        } else {
                            p.res[v] = r;
                        }
                    }
                    const double q1 = want ? one_m_a * r : 0.0;
                    if (p.qd && q1 != q0) p.qd[v] = q1;
                }
                stage_push(fst, out, want, (int)v, deg, 0.f, r);
                list_push(p.dangle, &ctl->dctr[nslot], (unsigned)p.V, flags, dang, (int)v);
            }
        }
        stage_flush(fst, out);
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tph, 1);
        ++cur;
    }
    if (gtid == 0) {
        ctl->iterations = iters;
        p.st->stamp_base = sbase + cur + 2;
    }
}

__global__ void res_to_float(const double* __restrict__ r, float* __restrict__ out, int V) {
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) out[v] = (float)r[v];
}

// Owner markers of a CSR: mark[t] = the largest v with row[v] <= t * 2^log_tile.
__global__ void csr_tile_markers(const int* __restrict__ row, int V, unsigned ntiles, int log_tile,
                                 int* __restrict__ mark) {
    const unsigned stride = gridDim.x * blockDim.x;
    for (unsigned t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += stride) {
        const long long e = (long long)t << log_tile;
        int lo = 0, hi = V;
        while (hi - lo > 1) {
            const int mid = lo + ((hi - lo) >> 1);
            if ((long long)row[mid] <= e)
                lo = mid;
            else
                hi = mid;
        }
        mark[t] = lo;
    }
}

// ---------------------------------------------------------------------------------------
// host side

int build_markers(c2g_graph* g, const int* row, int** out) {
    const unsigned ntiles = (unsigned)(((size_t)g->E + (1u << kPullTileLog) - 1) >> kPullTileLog) + 1;
    C2G_CUDA(cudaMalloc(out, sizeof(int) * ntiles));
    csr_tile_markers<<<g->num_sms * 4, 256, 0, g->stream>>>(row, g->V, ntiles, kPullTileLog, *out);
    C2G_CUDA(cudaGetLastError());
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    return C2G_OK;
}

static int ppr_geometry(c2g_graph* g) {
    if (g->geom_ppr.blocks > 0) return C2G_OK;
    int coop = 0;
    C2G_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device));
    if (!coop) return fail(C2G_ERR_UNSUPPORTED, "device %d lacks cooperative launch", g->device);
    int per_sm = 0;
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ppr_persistent, kPprThreads, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "PPR kernel cannot be resident (occupancy 0)");
    g->geom_ppr.blocks = per_sm * g->num_sms;
    g->geom_ppr.threads = kPprThreads;
    return C2G_OK;
}

void ppr_free(c2g_graph* g) {
    PprWork& w = g->ppr;
    void* ptrs[] = {w.pr, w.res, w.msg, w.qd, w.res_f, w.stamp, w.q[0], w.q[1], w.qval[0], w.qval[1],
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
    C2G_CUDA(cudaMalloc(&w.res, sizeof(double) * nv));
    C2G_CUDA(cudaMalloc(&w.msg, sizeof(double) * nv));
    C2G_CUDA(cudaMalloc(&w.qd, sizeof(double) * nv));
    C2G_CUDA(cudaMalloc(&w.res_f, sizeof(float) * nv));
    C2G_CUDA(cudaMalloc(&w.stamp, sizeof(int) * nv));
    C2G_CUDA(cudaMalloc(&w.touched, sizeof(int) * nv));
    C2G_CUDA(cudaMalloc(&w.dangle, sizeof(int) * nv));
    for (int b = 0; b < 2; ++b) {
        C2G_CUDA(cudaMalloc(&w.q[b], sizeof(int2) * nv));
        C2G_CUDA(cudaMalloc(&w.qval[b], sizeof(double) * nv));
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

int build_reverse_graph(c2g_graph* g);

int ppr_launch_view(c2g_graph* g, const int32_t* row, const int2* adj, const int32_t* row_rev, const int2* adj_rev,
                    const int32_t* mark_rev, int32_t source, const c2g_ppr_params& pp, float absorb, int32_t n_src,
                    const int32_t* src_list, const float* src_r0, const int32_t* seed_v, const float* seed_w,
                    int32_t n_rec, float* pr_dev, float* res_dev, float* ms) {
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
    p.row_r = row_rev;
    p.adj_r = adj_rev;
    p.mark_r = mark_rev;
    p.pull_div = row_rev ? g->ppr_cfg.pull_div : 0;
    p.dense_div = g->ppr_cfg.dense_div;
    p.pr = pr_dev ? pr_dev : w.pr;
    p.res = w.res;
    p.msg = w.msg;
    p.qd = w.qd;
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
    p.barrier_ns = g->barrier_ns ? g->barrier_ns : 2000000000ull;
    C2G_CUDA(cudaMemsetAsync(w.ctl, 0, sizeof(TraversalCtl), g->stream));
    void* args[] = {&p};
    C2G_CUDA(cudaEventRecord(g->ev0, g->stream));
    C2G_CUDA(cudaLaunchCooperativeKernel((const void*)ppr_persistent, dim3(g->geom_ppr.blocks),
                                         dim3(g->geom_ppr.threads), args, 0, g->stream));
    C2G_CUDA(cudaEventRecord(g->ev1, g->stream));
    // FP64 residuals reach the caller as float.
    res_to_float<<<g->num_sms * 4, 256, 0, g->stream>>>(w.res, res_dev ? res_dev : w.res_f, g->V);
    C2G_CUDA(cudaGetLastError());
    if (ms) {
        C2G_CUDA(cudaEventSynchronize(g->ev1));
        C2G_CUDA(cudaEventElapsedTime(ms, g->ev0, g->ev1));
    }
    return C2G_OK;
}

int ppr_launch(c2g_graph* g, int32_t source, const c2g_ppr_params& pp, const int32_t* seed_v,
               const float* seed_w, int32_t n_rec, float* pr_dev, float* res_dev, float* ms) {
    const int32_t* row_r = nullptr;
    const int2* adj_r = nullptr;
    const int32_t* mark_r = nullptr;
    if (!g->adj_f) return fail(C2G_ERR_UNSUPPORTED, "graph has no float weights (flist)");
    if (g->ppr_cfg.pull_div > 0) {
        int rc = build_reverse_graph(g);
        if (rc) return rc;
        row_r = g->row_r;
        adj_r = g->adj_r;
        mark_r = g->mark_r;
    }
    return ppr_launch_view(g, g->row, g->adj_f, row_r, adj_r, mark_r, source, pp, pp.alpha, 0, nullptr, nullptr,
                           seed_v, seed_w, n_rec, pr_dev, res_dev, ms);
}

}  // namespace c2g
