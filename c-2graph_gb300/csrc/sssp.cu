// Single-query SSSP for sm_103a: one persistent cooperative launch per query.
//
// Replaces CalcuSSSP (reference src/sssp/base/Main.cu:109-356 and
// src/sssp/purn/Main.cu:136-393).  Same result: the int32 shortest-distance fixed point
// of dis[source] = 0 plus the pruned-record seeds (sssp-purn), unreachable = 1999999999.
// Different schedule:
//   * frontier = sparse list of (vertex, edge base) appended by warp-aggregated atomics
//     when a distance improves (no O(V) isactive sweep, src/sssp/purn/Main.cu:350-377);
//   * expansion is edge-tiled: the frontier's out-edges form one index range [0, T),
//     each warp takes tiles of 2^log_tile edges from a dynamic counter, so low-degree
//     vertices share a tile (thread-per-edge), high-degree vertices span many tiles
//     (many warps per vertex), and every lane reads consecutive (target, weight) pairs;
//   * relaxation is an L2 read guarding int32 atomicMin (src/sssp/purn/Main.cu:257-260);
//   * optional near/far split (delta-stepping): improvements at or above the bucket
//     threshold go to a far pile that is filtered into the frontier when the near
//     frontier runs dry;
//   * one bounded grid barrier per round instead of four unbounded spins.
#include <climits>
#include <cstring>
#include <mutex>

#include "device_common.cuh"
#include "internal.h"

namespace c2g {

struct SsspParams {
    const int* row;
    const int2* adj;
    unsigned E;
    int V;
    int* dist;
    int* stamp;
    int* farstamp;
    int stamp_extent;  // entries of stamp/farstamp cleared when the round tags restart (>= V)
    int2* q[2];
    int* mark[2];
    int* far[3];
    TraversalCtl* ctl;
    StampState* st;
    int source;
    const int* seed_v;
    const int* seed_w;
    int n_seeds;
    int delta;
    int log_tile;
    int max_iter;
    unsigned mark_cap;
    unsigned long long barrier_ns;
    unsigned bar_extra;  // > 0: barriers wait for blocks that do not exist (watchdog test)
};

__device__ __forceinline__ FrontierOut sssp_out(const SsspParams& p, int buf, int slot) {
    FrontierOut o;
    o.q = p.q[buf];
    o.val = nullptr;
    o.mark = p.mark[buf];
    o.ctr = &p.ctl->qctr[slot];
    o.cap = (unsigned)p.V;
    o.mark_cap = p.mark_cap;
    o.log_tile = p.log_tile;
    o.flags = &p.ctl->flags;
    return o;
}

// Near-frontier candidate: dedup by round tag, drop vertices without out-edges.
__device__ __forceinline__ bool claim_near(const SsspParams& p, int c, int tag, int& deg) {
    if (ldcg(p.stamp + c) == tag || atomicExch(p.stamp + c, tag) == tag) return false;
    deg = __ldg(p.row + c + 1) - __ldg(p.row + c);
    return deg > 0;
}

// Far pile stage of one warp: staged ids plus the minimum distance staged so far.
struct FarStage {
    WarpStage st;
    int fmin;
};

// Warp-collective: stage lanes with `want` for far pile fb (deduplicated per epoch when
// `dedup`), tracking the minimum pushed distance.
__device__ __forceinline__ void far_stage(const SsspParams& p, FarStage& fs, int fb, bool want, int c, int d,
                                          int epoch, bool dedup) {
    if (want && dedup) {
        if (ldcg(p.farstamp + c) == epoch || atomicExch(p.farstamp + c, epoch) == epoch) want = false;
    }
    if (__ballot_sync(kFull, want) == 0) return;
    int mn = want ? d : INT_MAX;
#pragma unroll
    for (int o = 16; o >= 1; o >>= 1) mn = min(mn, __shfl_xor_sync(kFull, mn, o));
    fs.fmin = min(fs.fmin, mn);
    list_stage_push(fs.st, p.far[fb], &p.ctl->farctr[fb], (unsigned)p.V, &p.ctl->flags, want, c);
}

__device__ __forceinline__ void far_flush(const SsspParams& p, FarStage& fs, int fb) {
    list_stage_flush(fs.st, p.far[fb], &p.ctl->farctr[fb], (unsigned)p.V, &p.ctl->flags);
    if ((threadIdx.x & 31) == 0 && fs.fmin != INT_MAX) atomicMin(&p.ctl->farmin[fb], fs.fmin);
    fs.fmin = INT_MAX;
}

constexpr int kSsspUnroll = 4;  // edges in flight per lane

template <bool kDelta>
__device__ __forceinline__ void sssp_expand(const SsspParams& p, int buf, unsigned F, unsigned T, int tag_next,
                                            int thresh, int fb, int epoch, const FrontierOut& nout,
                                            WarpStage& fst, FarStage& far) {
    constexpr int U = kSsspUnroll;
    walk_frontier_edges<U>(
        p.q[buf], p.mark[buf], p.row, F, T, p.log_tile, p.mark_cap, (unsigned)p.V, p.E, &p.ctl->flags,
        [&](int v, unsigned) { return ldcg(p.dist + v); },  // snapshot distance of the owner
        [&](const bool* ok, const unsigned* idx, const int* du) {
            int c[U], nd[U], cur[U];
            // U independent edge loads, then U independent distance reads.
#pragma unroll
            for (int u = 0; u < U; ++u) {
                const int2 ew = ok[u] ? __ldg(p.adj + idx[u]) : make_int2(0, 0);
                c[u] = ew.x;
                nd[u] = du[u] + ew.y;
            }
#pragma unroll
            for (int u = 0; u < U; ++u) cur[u] = ok[u] ? ldcg(p.dist + c[u]) : INT_MIN;
            bool near[U], farp[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                near[u] = farp[u] = false;
                if (nd[u] < cur[u]) {  // an L2 read guards the atomic
                    const int old = atomicMin(p.dist + c[u], nd[u]);
                    if (nd[u] < old) {
                        if (!kDelta || nd[u] < thresh)
                            near[u] = true;
                        else
                            farp[u] = true;
                    }
                }
            }
#pragma unroll
            for (int u = 0; u < U; ++u) {
                int deg = 0;
                const bool want = near[u] && claim_near(p, c[u], tag_next, deg);
                stage_push(fst, nout, want, c[u], deg, 0.f);
                if (kDelta) far_stage(p, far, fb, farp[u], c[u], nd[u], epoch, true);
            }
        });
    stage_flush(fst, nout);
    if (kDelta) far_flush(p, far, fb);
}

template <bool kDelta>
__global__ void __launch_bounds__(512, 2) sssp_persistent(const SsspParams p) {
    TraversalCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned gwarp = gtid >> 5, nwarps = nthreads >> 5;
    const unsigned V = (unsigned)p.V;
    __shared__ StageSmem sm;
    const int wib = threadIdx.x >> 5;
    WarpStage fst{sm.v0[wib], sm.d0[wib], nullptr, 0};
    FarStage far{WarpStage{sm.v1[wib], nullptr, nullptr, 0}, INT_MAX};
    unsigned long long tph = globaltimer_ns();

    int sbase = p.st->stamp_base;
    int ebase = p.st->epoch_base;
    const bool reset = sbase > (1 << 29) || ebase > (1 << 29);
    if (reset) sbase = ebase = 0;

    // Init: dis = INF (src/sssp/purn/Main.cu:144-156).
    for (unsigned v = gtid; v < V; v += nthreads) p.dist[v] = kInfDist;
    // Restarting tags clear every stamp the array holds, not only this graph's V: an
    // array shared by calls on graphs of different sizes keeps older tags beyond V,
    // which a later, larger graph would read as current.
    if (reset)
        for (unsigned v = gtid; v < (unsigned)p.stamp_extent; v += nthreads) {
            p.stamp[v] = -1;
            p.farstamp[v] = -1;
        }
    if (gtid == 0) ctl->farmin[0] = ctl->farmin[1] = ctl->farmin[2] = INT_MAX;
    if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;

    // Source and pruned-record seeds (src/sssp/purn/Main.cu:160-181).
    if (gtid == 0) {
        atomicMin(p.dist + p.source, 0);
        ctl->seeds = p.n_seeds;
    }
    for (unsigned i = gtid; i < (unsigned)p.n_seeds; i += nthreads) atomicMin(p.dist + p.seed_v[i], p.seed_w[i]);
    if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;

    // Round-1 frontier: the seeds and the source, deduplicated.
    {
        const int tag = sbase + 1;
        const FrontierOut out = sssp_out(p, 1, 1);
        const unsigned n = (unsigned)p.n_seeds + 1;
        for (unsigned b = gwarp * 32; b < n; b += nwarps * 32) {
            const unsigned i = b + (unsigned)lane;
            bool want = false;
            int v = 0, deg = 0;
            if (i < n) {
                v = (i < (unsigned)p.n_seeds) ? p.seed_v[i] : p.source;
                want = claim_near(p, v, tag, deg);
            }
            stage_push(fst, out, want, v, deg, 0.f);
        }
        stage_flush(fst, out);
    }
    if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;
    phase_mark(ctl->phase_ns, tph, 0);

    int cur = 1, fb = 0, epoch = ebase + 1, iters = 0;
    int thresh = kDelta ? p.delta : INT_MAX;
    for (;;) {
        const unsigned long long c = ldcg(&ctl->qctr[cur % 3]);
        const unsigned F = (unsigned)(c >> 32), T = (unsigned)c;
        if (F == 0) {
            if (!kDelta) break;
            const unsigned fc = ldcg(&ctl->farctr[fb]);
            if (fc == 0) break;
            // Next bucket: at least thresh + delta, and past the far pile's minimum.
            const int fm = ldcg(&ctl->farmin[fb]);
            long long nt = (long long)thresh + p.delta;
            const long long jump = ((long long)fm / p.delta + 1) * (long long)p.delta;
            if (jump > nt) nt = jump;
            if (nt > INT_MAX) nt = INT_MAX;
            const int fdst = (fb + 1) % 3;
            if (gtid == 0) {
                const int fold = (fb + 2) % 3;  // read by the previous filter, free now
                ctl->farctr[fold] = 0;
                ctl->farmin[fold] = INT_MAX;
                ctl->qctr[(cur + 2) % 3] = 0ull;
                ctl->tilectr[(cur + 2) % 3] = 0u;
            }
            // The filter's frontier is the next round's (slot cur + 1): every thread has
            // read slot cur above to see it empty, and a late reader must not see these
            // appends there (it would take the expansion branch and skip its share of
            // the pile).
            const FrontierOut out = sssp_out(p, (cur + 1) & 1, (cur + 1) % 3);
            const int tag = sbase + cur + 1;
            for (unsigned b = gwarp * 32; b < fc; b += nwarps * 32) {
                const unsigned i = b + (unsigned)lane;
                bool near = false, keep = false;
                int v = 0, deg = 0, d = 0;
                if (i < fc) {
                    v = ldcg(p.far[fb] + i);
                    d = ldcg(p.dist + v);
                    if (d >= thresh) {
                        if (d < (int)nt)
                            near = claim_near(p, v, tag, deg);
                        else {
                            keep = true;
                            p.farstamp[v] = epoch + 1;
                        }
                    }
                }
                stage_push(fst, out, near, v, deg, 0.f);
                far_stage(p, far, fdst, keep, v, d, epoch + 1, false);
            }
            stage_flush(fst, out);
            far_flush(p, far, fdst);
            thresh = (int)nt;
            fb = fdst;
            ++epoch;
            if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;
            phase_mark(ctl->phase_ns, tph, 1);
            ++cur;
            continue;
        }
        if (++iters > p.max_iter) {
            if (gtid == 0) atomicOr(flags, C2G_FLAG_ITER_CAP);
            break;
        }
        if (gtid == 0) {
            ctl->qctr[(cur + 2) % 3] = 0ull;
            ctl->tilectr[(cur + 2) % 3] = 0u;
            ctl->popped += F;
            ctl->relaxed += T;
        }
        const FrontierOut nout = sssp_out(p, (cur + 1) & 1, (cur + 1) % 3);
        sssp_expand<kDelta>(p, cur & 1, F, T, sbase + cur + 1, thresh, fb, epoch, nout, fst, far);
        if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;
        phase_mark(ctl->phase_ns, tph, 2);
        ++cur;
    }
    if (gtid == 0) {
        ctl->iterations = iters;
        p.st->stamp_base = sbase + cur + 2;
        p.st->epoch_base = epoch + 2;
    }
}

// Bellman-Ford rounds (delta = 0) with a bitmap next frontier.  A relaxation that
// improves a distance issues red.min on it and red.or of the vertex's bit into a
// V-bit map; neither waits for a return value, so the relaxation path has no atomic
// round trip (the list kernel above needs the atomicMin result and a round-tag exchange
// per improved vertex).  A sweep over the V/32 map words then builds the next frontier
// in vertex order (entries, edge-base prefix, tile markers) and clears the words:
// two grid barriers per round instead of one.
constexpr int kSweepGroup = 4;  // map words whose row bounds are loaded together
constexpr int kBitsThreads = 512;  // block size of the bitmap kernel (its own launch geometry)
constexpr int kBitsBlocksPerSm = 2;
// Round-robin tiles in the expansion: a dynamic tile queue measured slower here (2.74 vs
// 2.20 ms per scale-22 query).
constexpr bool kBitsDynTiles = false;

__device__ __forceinline__ void bits_sweep(const SsspParams& p, unsigned* bits, const FrontierOut& out,
                                           WarpStage& fst, unsigned gwarp, unsigned nwarps, int lane) {
    const unsigned V = (unsigned)p.V;
    const unsigned nw = (V + 31u) >> 5;
    for (unsigned b = gwarp * 32u; b < nw; b += nwarps * 32u) {
        const unsigned wi = b + (unsigned)lane;
        const unsigned m = wi < nw ? ldcg(bits + wi) : 0u;
        if (m) bits[wi] = 0u;
        unsigned nz = __ballot_sync(kFull, m != 0u);
        while (nz) {
            int ks[kSweepGroup], deg[kSweepGroup];
            bool set[kSweepGroup];
#pragma unroll
            for (int u = 0; u < kSweepGroup; ++u) {
                ks[u] = nz ? __ffs(nz) - 1 : -1;
                nz &= nz - 1u;
            }
#pragma unroll
            for (int u = 0; u < kSweepGroup; ++u) {
                const unsigned mk = ks[u] < 0 ? 0u : (unsigned)__shfl_sync(kFull, (int)m, ks[u] < 0 ? 0 : ks[u]);
                const unsigned v = ((b + (unsigned)(ks[u] < 0 ? 0 : ks[u])) << 5) + (unsigned)lane;
                set[u] = (mk >> lane) & 1u;
                deg[u] = set[u] ? __ldg(p.row + v + 1) - __ldg(p.row + v) : 0;
            }
#pragma unroll
            for (int u = 0; u < kSweepGroup; ++u) {
                if (ks[u] < 0) break;  // warp-uniform
                const unsigned v = ((b + (unsigned)ks[u]) << 5) + (unsigned)lane;
                stage_push(fst, out, set[u] && deg[u] > 0, (int)v, deg[u], 0.f);
            }
        }
    }
    stage_flush(fst, out);
}

__global__ void __launch_bounds__(kBitsThreads, kBitsBlocksPerSm) sssp_bits_persistent(const SsspParams p,
                                                                                       unsigned* bits) {
    TraversalCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned gwarp = gtid >> 5, nwarps = nthreads >> 5;
    const unsigned V = (unsigned)p.V;
    __shared__ StageSmem sm;
    const int wib = threadIdx.x >> 5;
    WarpStage fst{sm.v0[wib], sm.d0[wib], nullptr, 0};
    unsigned long long tph = globaltimer_ns();

    // Init: dis = INF (src/sssp/purn/Main.cu:144-156), empty map.
    for (unsigned v = gtid; v < V; v += nthreads) p.dist[v] = kInfDist;
    for (unsigned i = gtid; i < ((V + 31u) >> 5); i += nthreads) bits[i] = 0u;
    if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;
    // Source and pruned-record seeds (src/sssp/purn/Main.cu:160-181) form round 1.
    if (gtid == 0) {
        atomicMin(p.dist + p.source, 0);
        atomicOr(bits + ((unsigned)p.source >> 5), 1u << (p.source & 31));
        ctl->seeds = p.n_seeds;
    }
    for (unsigned i = gtid; i < (unsigned)p.n_seeds; i += nthreads) {
        const int v = p.seed_v[i];
        atomicMin(p.dist + v, p.seed_w[i]);
        atomicOr(bits + ((unsigned)v >> 5), 1u << (v & 31));
    }
    if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;
    phase_mark(ctl->phase_ns, tph, 0);

    int cur = 1, iters = 0;
    for (;;) {
        const int buf = cur & 1, slot = cur % 3;
        if (gtid == 0) {
            ctl->qctr[(cur + 1) % 3] = 0ull;
            ctl->tilectr[(cur + 1) % 3] = 0u;
        }
        bits_sweep(p, bits, sssp_out(p, buf, slot), fst, gwarp, nwarps, lane);
        if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;
        phase_mark(ctl->phase_ns, tph, 1);
        const unsigned long long c = ldcg(&ctl->qctr[slot]);
        const unsigned F = (unsigned)(c >> 32), T = (unsigned)c;
        if (F == 0) break;
        if (++iters > p.max_iter) {
            if (gtid == 0) atomicOr(flags, C2G_FLAG_ITER_CAP);
            break;
        }
        if (gtid == 0) {
            ctl->popped += F;
            ctl->relaxed += T;
        }
        constexpr int U = kSsspUnroll;
        walk_frontier_edges<U>(
            p.q[buf], p.mark[buf], p.row, F, T, p.log_tile, p.mark_cap, V, p.E, flags,
            [&](int v, unsigned) { return ldcg(p.dist + v); },  // the owner's current distance
            [&](const bool* ok, const unsigned* idx, const int* du) {
                int c2[U], nd[U], cd[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int2 ew = ok[u] ? __ldg(p.adj + idx[u]) : make_int2(0, 0);
                    c2[u] = ew.x;
                    nd[u] = du[u] + ew.y;
                }
#pragma unroll
                for (int u = 0; u < U; ++u) cd[u] = ok[u] ? ldcg(p.dist + c2[u]) : INT_MIN;
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    if (nd[u] < cd[u]) {  // an L2 read guards the update
                        atomicMin(p.dist + c2[u], nd[u]);
                        atomicOr(bits + ((unsigned)c2[u] >> 5), 1u << (c2[u] & 31));
                    }
                }
            },
            kBitsDynTiles ? &ctl->tilectr[slot] : nullptr);
        if (!grid_sync(bar, flags, p.barrier_ns, p.bar_extra)) return;
        phase_mark(ctl->phase_ns, tph, 2);
        ++cur;
    }
    if (gtid == 0) ctl->iterations = iters;
}

// ---------------------------------------------------------------------------------------
// host side

static int sssp_geometry(c2g_graph* g) {
    if (g->geom_sssp.blocks > 0) return C2G_OK;
    int coop = 0;
    C2G_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device));
    if (!coop) return fail(C2G_ERR_UNSUPPORTED, "device %d lacks cooperative launch", g->device);
    int per_sm_a = 0, per_sm_b = 0, per_sm_c = 0;
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_a, sssp_persistent<false>, 512, 0));
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_b, sssp_persistent<true>, 512, 0));
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_c, sssp_bits_persistent, kBitsThreads, 0));
    const int per_sm = per_sm_a < per_sm_b ? per_sm_a : per_sm_b;
    if (per_sm < 1 || per_sm_c < 1) return fail(C2G_ERR_CUDA, "SSSP kernel cannot be resident (occupancy 0)");
    g->geom_sssp.blocks = per_sm * g->num_sms;
    g->geom_sssp.threads = 512;
    g->geom_bits.blocks = per_sm_c * g->num_sms;
    g->geom_bits.threads = kBitsThreads;
    return C2G_OK;
}

void sssp_free(c2g_graph* g) {
    SsspWork& w = g->sssp;
    void* ptrs[] = {w.dist, w.stamp, w.farstamp, w.q[0], w.q[1], w.mark[0], w.mark[1],
                    w.far, w.bits, w.ctl, w.st};
    for (void* ptr : ptrs)
        if (ptr) cudaFree(ptr);
    w = SsspWork();
}

static int sssp_alloc(c2g_graph* g) {
    SsspWork& w = g->sssp;
    const int log_tile = g->sssp_cfg.log_tile;
    if (w.dist && w.log_tile == log_tile) return C2G_OK;
    if (w.dist) sssp_free(g);
    const size_t V = (size_t)g->V;
    const size_t nv = V ? V : 1;
    const unsigned mark_cap = (unsigned)(((size_t)g->E >> log_tile) + 2);
    C2G_CUDA(cudaMalloc(&w.dist, sizeof(int) * nv));
    C2G_CUDA(cudaMalloc(&w.stamp, sizeof(int) * nv));
    C2G_CUDA(cudaMalloc(&w.farstamp, sizeof(int) * nv));
    for (int b = 0; b < 2; ++b) {
        C2G_CUDA(cudaMalloc(&w.q[b], sizeof(int2) * nv));
        C2G_CUDA(cudaMalloc(&w.mark[b], sizeof(int) * mark_cap));
    }
    C2G_CUDA(cudaMalloc(&w.far, sizeof(int) * nv * 3));
    C2G_CUDA(cudaMalloc(&w.bits, sizeof(unsigned) * ((nv + 31) / 32)));
    C2G_CUDA(cudaMalloc(&w.ctl, sizeof(TraversalCtl)));
    C2G_CUDA(cudaMalloc(&w.st, sizeof(StampState)));
    C2G_CUDA(cudaMemsetAsync(w.stamp, 0xff, sizeof(int) * nv, g->stream));
    C2G_CUDA(cudaMemsetAsync(w.farstamp, 0xff, sizeof(int) * nv, g->stream));
    C2G_CUDA(cudaMemsetAsync(w.st, 0, sizeof(StampState), g->stream));
    w.mark_cap = mark_cap;
    w.log_tile = log_tile;
    return C2G_OK;
}

int sssp_launch(c2g_graph* g, int32_t source, const int32_t* seed_v, const int32_t* seed_w, int32_t n_seeds,
                int32_t* dist_dev, float* ms) {
    int rc;
    if ((rc = sssp_geometry(g))) return rc;
    if ((rc = sssp_alloc(g))) return rc;
    if (!g->adj_w) return fail(C2G_ERR_UNSUPPORTED, "graph has no int32 weights (wlist)");
    SsspWork& w = g->sssp;
    SsspParams p;
    p.row = g->row;
    p.adj = g->adj_w;
    p.V = g->V;
    p.E = (unsigned)g->E;
    p.dist = dist_dev ? dist_dev : w.dist;
    p.stamp = w.stamp;
    p.farstamp = w.farstamp;
    p.stamp_extent = g->V;
    p.q[0] = w.q[0];
    p.q[1] = w.q[1];
    p.mark[0] = w.mark[0];
    p.mark[1] = w.mark[1];
    const size_t nv = g->V ? (size_t)g->V : 1;
    p.far[0] = w.far;
    p.far[1] = w.far + nv;
    p.far[2] = w.far + 2 * nv;
    p.ctl = w.ctl;
    p.st = w.st;
    p.source = source;
    p.seed_v = seed_v;
    p.seed_w = seed_w;
    p.n_seeds = n_seeds;
    p.delta = g->sssp_cfg.delta;
    p.log_tile = w.log_tile;
    p.max_iter = g->sssp_cfg.max_iter;
    p.mark_cap = w.mark_cap;
    p.barrier_ns = g->barrier_ns ? g->barrier_ns : 2000000000ull;
    p.bar_extra = g->stall_next_sssp ? 1u : 0u;
    g->stall_next_sssp = 0;
    C2G_CUDA(cudaMemsetAsync(w.ctl, 0, sizeof(TraversalCtl), g->stream));
    unsigned* bits = w.bits;
    void* args[] = {&p, &bits};
    const bool delta = p.delta > 0;
    // delta = 0: Bellman-Ford rounds with the bitmap frontier; delta > 0: near/far buckets
    C2G_CUDA(cudaEventRecord(g->ev0, g->stream));
    C2G_CUDA(cudaLaunchCooperativeKernel(delta ? (const void*)sssp_persistent<true> : (const void*)sssp_bits_persistent,
                                         dim3(delta ? g->geom_sssp.blocks : g->geom_bits.blocks),
                                         dim3(delta ? g->geom_sssp.threads : g->geom_bits.threads), args, 0, g->stream));
    C2G_CUDA(cudaEventRecord(g->ev1, g->stream));
    if (ms) {
        C2G_CUDA(cudaEventSynchronize(g->ev1));
        C2G_CUDA(cudaEventElapsedTime(ms, g->ev0, g->ev1));
    }
    return C2G_OK;
}

}  // namespace c2g

// ---------------------------------------------------------------------------------------
// Allocation-free entry point.
//
// Some callers cannot let this library allocate device memory per call.  Examples are a
// host whose device memory is owned entirely by another allocator, and a serving loop
// that must not call cudaMalloc/cudaFree after start-up (both may synchronise the device
// and stall every stream).  c2g_sssp_noalloc runs the same single-query kernel as
// c2g_sssp on arrays the caller already holds on the device.  Its scratch memory
// (round tags, frontier queues, tile markers and the launch control block) is
// g_sssp_noalloc_scratch below: a fixed array, loaded with the library on every GPU that
// uses it and held until the process exits.  Its size bounds the graphs this entry
// point accepts (C2G_NOALLOC_MAX_V vertices, C2G_NOALLOC_MAX_E edges).

namespace c2g {
namespace {

constexpr int kNoAllocLogTile = 8;
constexpr size_t kNoAllocMarks = ((size_t)C2G_NOALLOC_MAX_E >> kNoAllocLogTile) + 2;

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }
constexpr size_t kOffStamp = 0;
constexpr size_t kOffFarstamp = kOffStamp + align256(sizeof(int) * (size_t)C2G_NOALLOC_MAX_V);
constexpr size_t kOffQ0 = kOffFarstamp + align256(sizeof(int) * (size_t)C2G_NOALLOC_MAX_V);
constexpr size_t kOffQ1 = kOffQ0 + align256(sizeof(int2) * (size_t)C2G_NOALLOC_MAX_V);
constexpr size_t kOffMark0 = kOffQ1 + align256(sizeof(int2) * (size_t)C2G_NOALLOC_MAX_V);
constexpr size_t kOffMark1 = kOffMark0 + align256(sizeof(int) * kNoAllocMarks);
constexpr size_t kOffCtl = kOffMark1 + align256(sizeof(int) * kNoAllocMarks);
constexpr size_t kOffSt = kOffCtl + align256(sizeof(TraversalCtl));
constexpr size_t kNoAllocScratchBytes = kOffSt + align256(sizeof(StampState));

constexpr int kNoAllocMaxDevices = 64;
void* g_noalloc_base[kNoAllocMaxDevices];  // device address of the scratch, per device (null: not looked up)
std::mutex g_noalloc_mu;

}  // namespace

// The scratch.  Zero at module load: round tags start above 0 and the tag bases start at
// 0, so no clearing is needed before the first call; the control block is cleared on the
// caller's stream before every launch.
static __device__ __align__(256) unsigned char g_sssp_noalloc_scratch[kNoAllocScratchBytes];

}  // namespace c2g

extern "C" int c2g_sssp_noalloc(const int32_t* row, const void* adj, int32_t V, int64_t E, int32_t source,
                                int32_t* dist, void* stream, c2g_stats* stats) {
    using namespace c2g;
    if (!row || !adj || !dist) return fail(C2G_ERR_ARG, "noalloc SSSP: NULL argument");
    if (V < 1 || V > C2G_NOALLOC_MAX_V)
        return fail(C2G_ERR_RANGE, "noalloc SSSP: V = %d outside [1, %d] (size of the static scratch)", V,
                    C2G_NOALLOC_MAX_V);
    if (E < 0 || E > C2G_NOALLOC_MAX_E)
        return fail(C2G_ERR_RANGE, "noalloc SSSP: E = %lld outside [0, %lld] (size of the static scratch)",
                    (long long)E, (long long)C2G_NOALLOC_MAX_E);
    if (source < 0 || source >= V) return fail(C2G_ERR_RANGE, "source %d out of range [0,%d)", source, V);
    int dev = 0;
    C2G_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= kNoAllocMaxDevices) return fail(C2G_ERR_UNSUPPORTED, "device index %d too large", dev);
    // Once per device, with that device current: the device address of the scratch.
    // The host-side name of a __device__ array is not a device address.  Only a
    // successful lookup is kept; a failed one (say, made during a stream capture) is
    // retried by the next call.
    unsigned char* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        if (!g_noalloc_base[dev]) {
            void* addr = nullptr;
            const cudaError_t e = cudaGetSymbolAddress(&addr, g_sssp_noalloc_scratch);
            if (e != cudaSuccess) {
                cudaGetLastError();
                return fail(C2G_ERR_CUDA, "noalloc SSSP: cudaGetSymbolAddress failed: %s", cudaGetErrorString(e));
            }
            g_noalloc_base[dev] = addr;
        }
        base = static_cast<unsigned char*>(g_noalloc_base[dev]);
    }
    cudaStream_t s = static_cast<cudaStream_t>(stream);

    int coop = 0, per_sm = 0, sms = 0;
    C2G_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, dev));
    if (!coop) return fail(C2G_ERR_UNSUPPORTED, "device %d lacks cooperative launch", dev);
    C2G_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sssp_persistent<false>, 512, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "SSSP kernel cannot be resident (occupancy 0)");

    SsspParams p;
    p.row = row;
    p.adj = static_cast<const int2*>(adj);
    p.E = (unsigned)E;
    p.V = V;
    p.dist = dist;
    p.stamp = reinterpret_cast<int*>(base + kOffStamp);
    p.farstamp = reinterpret_cast<int*>(base + kOffFarstamp);
    p.stamp_extent = C2G_NOALLOC_MAX_V;  // the array serves graphs of every size
    p.q[0] = reinterpret_cast<int2*>(base + kOffQ0);
    p.q[1] = reinterpret_cast<int2*>(base + kOffQ1);
    p.mark[0] = reinterpret_cast<int*>(base + kOffMark0);
    p.mark[1] = reinterpret_cast<int*>(base + kOffMark1);
    p.far[0] = p.far[1] = p.far[2] = nullptr;  // the near/far split is off here
    p.ctl = reinterpret_cast<TraversalCtl*>(base + kOffCtl);
    p.st = reinterpret_cast<StampState*>(base + kOffSt);
    p.source = source;
    p.seed_v = nullptr;
    p.seed_w = nullptr;
    p.n_seeds = 0;
    p.delta = 0;
    p.log_tile = kNoAllocLogTile;
    p.max_iter = 1 << 20;
    p.mark_cap = (unsigned)(((size_t)E >> kNoAllocLogTile) + 2);
    p.barrier_ns = 2000000000ull;
    p.bar_extra = 0u;
    C2G_CUDA(cudaMemsetAsync(p.ctl, 0, sizeof(TraversalCtl), s));
    void* args[] = {&p};
    C2G_CUDA(cudaLaunchCooperativeKernel((const void*)sssp_persistent<false>, dim3(per_sm * sms), dim3(512), args, 0,
                                         s));
    TraversalCtl ctl;
    C2G_CUDA(cudaMemcpyAsync(&ctl, p.ctl, sizeof(ctl), cudaMemcpyDeviceToHost, s));
    C2G_CUDA(cudaStreamSynchronize(s));
    if (ctl.flags & (C2G_FLAG_BARRIER_TIMEOUT | C2G_FLAG_QUEUE_OVERFLOW | C2G_FLAG_BOUNDS)) {
        static const StampState reset{1 << 30, 1 << 30, {0, 0}};
        cudaMemcpyAsync(p.st, &reset, sizeof(reset), cudaMemcpyHostToDevice, s);
        cudaStreamSynchronize(s);
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->source = source;
        stats->iterations = ctl.iterations;
        stats->vertices_popped = ctl.popped;
        stats->edges_relaxed = ctl.relaxed;
        stats->status_flags = ctl.flags;
        stats->alg_bytes = 4.0 * V + 16.0 * (double)ctl.popped + 12.0 * (double)ctl.relaxed;
    }
    if (ctl.flags & C2G_FLAG_BARRIER_TIMEOUT) return fail(C2G_ERR_TIMEOUT, "grid barrier wait ran out");
    if (ctl.flags & (C2G_FLAG_QUEUE_OVERFLOW | C2G_FLAG_BOUNDS))
        return fail(C2G_ERR_OVERFLOW, "device queue or index check failed");
    return C2G_OK;
}
