// Batched multi-query SSSP for sm_103a: up to thousands of sources in ONE persistent
// cooperative launch, with per-query bitmask frontiers.
//
// The reference runs one query per launch (src/sssp/purn/Main.cu:67-99) and, in its
// PM mode, two queries on two streams (src/sssp/purn-perk/Main.cu:51-53,107,164).  Here
// Q queries (padded to a multiple of 32) share every pass over the graph:
//   * state is vertex-major: dist[v][Q] int32, so the 32 queries of one "word" w of a
//     vertex occupy one 128-byte line;
//   * a frontier entry is a (vertex, word) pair with a 32-bit mask of the word's queries
//     that improved the vertex in the previous round;
//   * expansion: a warp reads 32 edges of an entry (one per lane) and broadcasts them;
//     for each edge every lane relaxes one query of the word with one coalesced
//     128-byte read of the target's row, so an edge read from HBM serves all active
//     queries of its word;
//   * an improvement is red.min on the distance and red.or of the query bits into the
//     target's (vertex, word) mask: nothing on the relaxation path waits for an atomic;
//   * a round is two phases: a sweep of the mask words that builds the frontier (with
//     edge-base prefix and tile markers), then the expansion.
// Results are the same int32 fixed points as one c2g_sssp call per source.
#include <climits>
#include <cmath>
#include <cstring>
#include <algorithm>
#include <vector>

#include "device_common.cuh"
#include "f32x2.h"
#include "fp64_mul.h"
#include "internal.h"

namespace c2g {

struct BatchParams {
    const int* row;
    const int2* adj;
    unsigned E;
    int V;
    int logW;  // words per vertex = 1 << logW
    int Q;     // padded query count = 32 << logW
    int nq;    // real queries
    int* dist;          // [V][Q]
    unsigned* mask;     // [V][W] next-round masks
    int2* q[2];         // entries (v*W + w, edge base)
    unsigned* qmask[2]; // gathered masks per entry
    int* mark[2];
    TraversalCtl* ctl;
    const int* sources;   // [nq]
    const int* seed_off;  // [nq+1] offsets into seed_v/seed_w (or nullptr)
    const int* seed_v;
    const int* seed_w;
    unsigned qcap;
    unsigned mark_cap;
    int max_iter;
    unsigned long long barrier_ns;
    long long* counters;  // [2]: relaxations (query, edge), edge-word steps
    int tile_big_log;     // log2 of the big tile's edge-word steps (>= kBatchTileLog)
    int tile_min_log;     // a round walks big tiles when it has >= 2^tile_min_log of them per warp
    int epoch_rounds;     // > 0: an epoch of a resident batch (no initialisation; at most this many rounds)
    RoundTrace* trace;    // [kMaxTraceRounds + 1] per-round trace
    // pull rounds: reverse CSR with int32 weights and its tile owners; a round pulls when its
    // (query, edge) relaxations exceed pull_min (~0: never); amask[b] holds the frontier's lanes per
    // (vertex, word) of the rounds of parity b (zero elsewhere)
    const int* row_r;
    const int2* adj_rw;
    const int* mark_r;
    unsigned ntiles_r;
    unsigned long long pull_min;
    unsigned* amask[2];
};

// A warp's chunk of up to 32 in-edges of a pull round (batched SSSP and PPR), staged in shared memory: source, weight bits and
// the source's active lanes in the item's 4 query words.  Each lane loads one in-edge and
// the live ones (a source with an active lane) are compacted into the chunk; the warp
// then reads them one by one as broadcasts (two shared loads per in-edge instead of six
// shuffles, and the chunk's values leave the registers of the gather loop).
struct PullChunk {
    int2 ed[32];
    uint4 mk[32];
};

// Warp tiles of the expansion: markers are laid every 2^kBatchTileLog edge-word steps; a
// round with enough work (at least 2^tile_min_log big tiles per warp) walks tiles of
// 2^tile_big_log steps (every 2^(big - kBatchTileLog)-th marker), a smaller one tiles of
// 2^kBatchTileLog.  The handle's defaults are big 512, at least 16 per warp (256 sources
// at scale 22: 132 ms per SSSP batch with 128-step tiles, 121 ms with 512; 32 sources at
// scale 20: 4.6 ms with 128, 5.4 ms with 512, too few tiles per warp);
// c2g_sssp_batch_autotune picks them per batch.
constexpr int kBatchTileLog = 7;

__device__ __forceinline__ int batch_tile_log(unsigned T, unsigned nwarps, int big, int min_log) {
    return big > kBatchTileLog && (unsigned long long)T >= ((unsigned long long)nwarps << (big + min_log))
               ? big
               : kBatchTileLog;
}

// The batched push walks big tiles of 512 steps in rounds with at least 16 per warp.
constexpr int kPushTileBig = 9;
constexpr int kPushTileMin = 4;

__device__ __forceinline__ void trace_round(RoundTrace* tr, int i, long long work, int shape) {
    if (i <= kMaxTraceRounds) tr[i] = RoundTrace{globaltimer_ns(), work, shape, 0u};
}

// The end of round i's first phase (right after its grid barrier).
__device__ __forceinline__ void trace_mid(RoundTrace* tr, int i) {
    if (i >= 0 && i <= kMaxTraceRounds) tr[i].mid_ns = (unsigned)(globaltimer_ns() - tr[i].t_ns);
}

__device__ __forceinline__ FrontierOut batch_out(const BatchParams& p, int buf, int slot) {
    FrontierOut o;
    o.q = p.q[buf];
    o.val = reinterpret_cast<float*>(p.qmask[buf]);  // mask bits travel in the value slot
    o.mark = p.mark[buf];
    o.ctr = &p.ctl->qctr[slot];
    o.cap = p.qcap;
    o.mark_cap = p.mark_cap;
    o.log_tile = kBatchTileLog;
    o.flags = &p.ctl->flags;
    return o;
}

// Build a round's frontier from the improvement masks: a sweep over all (vertex, word)
// mask words; each non-zero word is cleared and, when the vertex has out-edges, becomes an
// entry (v * W + w, edge base) carrying the mask.  Entries come out in sweep order per
// warp.  Relaxations set masks with fire-and-forget red.or, so no relaxation waits on an
// atomic's return; the sweep reads V * W words per round.
__device__ __forceinline__ void batch_sweep(const BatchParams& p, const FrontierOut& out, unsigned* am,
                                            unsigned long long* pcount, WarpStage& fst, unsigned gwarp,
                                            unsigned nwarps, int lane) {
    const unsigned nm = (unsigned)p.V << p.logW;
    unsigned long long rel = 0;  // (query, edge) relaxations of the frontier
    for (unsigned b = gwarp * 32u; b < nm; b += nwarps * 32u) {
        const unsigned i = b + (unsigned)lane;
        unsigned m = 0u;
        int deg = 0;
        if (i < nm) {
            m = ldcg(p.mask + i);
            if (m) {
                p.mask[i] = 0u;
                const int v = (int)(i >> p.logW);
                deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
            }
        }
        if (am && m != 0u && deg > 0) {
            am[i] = m;  // the pull rounds' lookup of the frontier's lanes
            rel += (unsigned long long)__popc(m) * (unsigned long long)deg;
        }
        stage_push(fst, out, m != 0u && deg > 0, (int)i, deg, __int_as_float((int)m));
    }
    stage_flush(fst, out);
    if (am) {
        for (int o = 16; o >= 1; o >>= 1) rel += __shfl_xor_sync(kFull, rel, o);
        if (lane == 0 && rel) atomicAdd(pcount, rel);
    }
}

constexpr int kBatchUnroll = 4;  // relaxation items in flight per lane
// Launch shape of the batched SSSP: 3 blocks of 384 threads per SM (36 warps) measured
// faster than 2 x 512 (32 warps) at the same 4 items per lane (132-135 vs 140 ms for 256
// sources at scale 22), 1 x 512 with 8-12 items (220 ms) and 6 x 256 (192 ms).
constexpr int kSsspBatchThreads = 384;


// Lane compaction of one owner run: the run's work is the items (edge ei, active-query
// slot j) for ei in [0, len) and j in [0, cnt), numbered i = ei * cnt + j; lane l takes
// items l, l + 32, l + 64, ... so every lane of a warp step relaxes something even when
// few of the word's 32 queries are active.  The (ei, j) of a lane advance by 32 items
// per step without a division (32 = dq * cnt + dr).  Lane 0 holds the lowest item, so
// the loop condition is warp-uniform; body(ei[U], j[U]) must check ei < len.
template <int U, typename Body>
__device__ __forceinline__ void owner_items(unsigned cnt, unsigned len, int lane, Body body) {
    const float rc = __frcp_rn((float)cnt);  // exact enough: (l + 0.5) / cnt is >= 1/64 from an integer
    int ei = (int)(((float)lane + 0.5f) * rc);
    int j = lane - ei * (int)cnt;
    const int dq = (int)(32.5f * rc);
    const int dr = 32 - dq * (int)cnt;
    while ((unsigned)__shfl_sync(kFull, ei, 0) < len) {
        int eis[U], js[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            eis[u] = ei;
            js[u] = j;
            ei += dq;
            j += dr;
            if (j >= (int)cnt) {
                j -= (int)cnt;
                ++ei;
            }
        }
        body(eis, js);
    }
}

// Pull round of the batched SSSP.  In a dense round (most (vertex, word) pairs improved in
// the previous round) the expansion reads a 128-byte distance line per edge-word step and
// issues red.min for every improvement.  A pull round walks the reverse CSR instead: for
// each target v and query word it takes the minimum of dist[u] + w over the in-edges
// u -> v whose source improved in the previous round (amask), lane by lane (lane = query),
// then compares it with dist[v]: a target whose in-edges lie in one tile gets plain
// stores of its improved lanes and of its next-round mask word; a target whose in-edges
// cross a tile boundary gets atomicMin / atomicOr.  Items are (tile of 2^kPullTileLog
// in-edges, group of 4 query words), in word-group-major order; a warp stages each chunk's
// live in-edges (a source with an active lane in the item's words) in shared memory, as
// the PPR pull does, and reads each live in-edge's source lines for the item's words.
// Any order of relaxations reaches the same fixed point, so the distances are those of
// the push rounds; pull and push rounds mix freely.
__device__ __forceinline__ void sbatch_pull(const BatchParams& p, int buf, unsigned* qctr, PullChunk& pc,
                                            long long& relax, int lane) {
    const unsigned W = 1u << p.logW;
    const int lg = p.logW >= 2 ? p.logW - 2 : 0;  // word groups per tile
    const unsigned nitems = p.ntiles_r << lg;
    const unsigned* am = p.amask[buf];
    const unsigned tw = 1u << kPullTileLog;
    const unsigned Qu = (unsigned)p.Q;
    unsigned itn = next_tile(qctr, lane);
    for (unsigned it = itn; it < nitems; it = itn) {
        itn = next_tile(qctr, lane);  // the next item, fetched while this one runs
        const unsigned t = it % p.ntiles_r;
        const unsigned w0 = (it / p.ntiles_r) * 4u;
        const unsigned e0 = t << kPullTileLog;
        const unsigned e1 = min(e0 + tw, p.E);
        int v = __ldg(p.mark_r + t);  // owner of in-edge e0
        unsigned vs = (unsigned)__ldg(p.row_r + v);
        for (;;) {
            const unsigned ve = (unsigned)__ldg(p.row_r + v + 1);
            const unsigned ea = max(vs, e0), ez = min(ve, e1);
            if (ea < ez) {  // warp-uniform: v has in-edges in this tile
                int mn[4] = {INT_MAX, INT_MAX, INT_MAX, INT_MAX};  // this lane's query in each word
                for (unsigned b = ea; b < ez; b += 32u) {
                    const unsigned e = b + (unsigned)lane;
                    int src = 0, wt = 0;
                    unsigned mk[4] = {0u, 0u, 0u, 0u};
                    if (e < ez) {
                        const int2 ed = __ldg(p.adj_rw + e);
                        if ((unsigned)ed.x >= (unsigned)p.V) {
                            atomicOr(&p.ctl->flags, C2G_FLAG_BOUNDS);
                        } else {
                            src = ed.x;
                            wt = ed.y;
                            const unsigned* ms = am + ((size_t)(unsigned)src << p.logW) + w0;
                            if (W >= 4u) {  // four words, 16-byte aligned
                                const uint4 m4 = ldcg(reinterpret_cast<const uint4*>(ms));
                                mk[0] = m4.x;
                                mk[1] = m4.y;
                                mk[2] = m4.z;
                                mk[3] = m4.w;
                            } else {
#pragma unroll
                                for (int j = 0; j < 4; ++j)
                                    if ((unsigned)j < W) mk[j] = ldcg(ms + j);
                            }
                        }
                    }
                    // (query, edge) relaxations of the chunk, counted by lane 0
                    const unsigned nrel = __reduce_add_sync(
                        kFull, (unsigned)(__popc(mk[0]) + __popc(mk[1]) + __popc(mk[2]) + __popc(mk[3])));
                    if (lane == 0) relax += (long long)nrel;
                    const bool live = (mk[0] | mk[1] | mk[2] | mk[3]) != 0u;
                    const unsigned lm = __ballot_sync(kFull, live);
                    const unsigned n = (unsigned)__popc(lm);
                    __syncwarp();  // the previous chunk's reads are done
                    if (live) {
                        const unsigned at = (unsigned)__popc(lm & ((1u << lane) - 1u));
                        pc.ed[at] = make_int2(src, wt);
                        pc.mk[at] = make_uint4(mk[0], mk[1], mk[2], mk[3]);
                    }
                    __syncwarp();
                    for (unsigned k = 0; k < n; ++k) {
                        // one in-edge's source lines, then its candidates (two in-edges in
                        // flight measured slower: 93.8 vs 90.2 ms per 256-query batch)
                        const int2 ek = pc.ed[k];
                        const uint4 mq = pc.mk[k];
                        int dv[4];
#pragma unroll
                        for (int j = 0; j < 4; ++j) {
                            const unsigned mj = j == 0 ? mq.x : j == 1 ? mq.y : j == 2 ? mq.z : mq.w;
                            // L2-coherent: other warps lower distances during the round
                            dv[j] = ((mj >> lane) & 1u)
                                        ? ldcg(p.dist + (size_t)(unsigned)ek.x * Qu + ((w0 + j) << 5) + lane)
                                        : INT_MAX;
                        }
#pragma unroll
                        for (int j = 0; j < 4; ++j)
                            if (dv[j] != INT_MAX) mn[j] = min(mn[j], dv[j] + ek.y);
                    }
                }
                const bool whole = vs >= e0 && ve <= e1;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    if (w0 + j >= W) break;  // warp-uniform
                    const size_t off = (size_t)(unsigned)v * Qu + ((w0 + j) << 5) + lane;
                    const unsigned vw = ((unsigned)v << p.logW) + w0 + (unsigned)j;
                    const bool imp = mn[j] != INT_MAX && mn[j] < ldcg(p.dist + off);
                    const unsigned bits = __ballot_sync(kFull, imp);
                    if (bits) {
                        if (whole) {  // this warp holds all of v's in-edges: no other writer
                            if (imp) p.dist[off] = mn[j];
                            if (lane == 0) p.mask[vw] = bits;
                        } else {
                            if (imp) atomicMin(p.dist + off, mn[j]);
                            if (lane == 0) atomicOr(p.mask + vw, bits);
                        }
                    }
                }
            }
            if (ve >= e1) break;
            ++v;
            vs = ve;
        }
    }
}

__global__ void __launch_bounds__(kSsspBatchThreads, 3) sssp_batch_persistent(const BatchParams p) {
    TraversalCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned gwarp = gtid >> 5, nwarps = nthreads >> 5;
    const int W = 1 << p.logW;
    const unsigned Qu = (unsigned)p.Q;
    __shared__ StageSmem sm;
    const int wib = threadIdx.x >> 5;
    unsigned long long tph = globaltimer_ns();
    WarpStage fst{sm.v0[wib], sm.d0[wib], sm.x0[wib], 0};
    int* qtab = sm.v1[wib];  // slot -> query position table of the owner being expanded
    __shared__ PullChunk pcs[kSsspBatchThreads / 32];  // pull rounds' in-edge chunks

    // An epoch of a resident batch starts from the state the previous epoch left: the
    // distances and the improvement masks (queries that joined since have their column
    // set and their source marked).
    if (p.epoch_rounds == 0) {
    // Init: dist = INF (vector stores), masks = 0.
    {
        const size_t n4 = ((size_t)p.V * (size_t)p.Q) >> 2;
        int4* d4 = reinterpret_cast<int4*>(p.dist);
        const int4 inf4 = make_int4(kInfDist, kInfDist, kInfDist, kInfDist);
        for (size_t i = gtid; i < n4; i += nthreads) d4[i] = inf4;
        const size_t nm = (size_t)p.V << p.logW;
        for (size_t i = gtid; i < nm; i += nthreads) p.mask[i] = 0u;
    }
    if (!grid_sync(bar, flags, p.barrier_ns)) return;

    // Sources and their seeds: dist[s][q] = 0, dist[seed][q] = min(w); mark them.  A warp
    // per query, its lanes over the seed records.
    for (unsigned qi = gwarp; qi < (unsigned)p.nq; qi += nwarps) {
        const int s = p.sources[qi];
        const unsigned bit = 1u << (qi & 31), w = qi >> 5;
        if (lane == 0) {
            atomicMin(p.dist + (size_t)s * p.Q + qi, 0);
            atomicOr(p.mask + ((size_t)s << p.logW) + w, bit);
        }
        if (p.seed_off)
            for (int k = p.seed_off[qi] + lane; k < p.seed_off[qi + 1]; k += 32) {
                atomicMin(p.dist + (size_t)p.seed_v[k] * p.Q + qi, p.seed_w[k]);
                atomicOr(p.mask + ((size_t)p.seed_v[k] << p.logW) + w, bit);
            }
    }
    if (!grid_sync(bar, flags, p.barrier_ns)) return;
    }
    phase_mark(ctl->phase_ns, tph, 0);

    long long relax = 0, steps = 0;
    int cur = 1, iters = 0;
    for (;;) {
        const int buf = cur & 1, slot = cur % 3;
        // Phase 1: this round's frontier from the masks of the previous one.
        if (gtid == 0) {
            ctl->qctr[(cur + 1) % 3] = 0ull;
            ctl->tilectr[(cur + 1) % 3] = 0u;
            ctl->pcount[(cur + 1) % 3] = 0ull;
        }
        batch_sweep(p, batch_out(p, buf, slot), p.pull_min != ~0ull ? p.amask[buf] : nullptr, &ctl->pcount[slot], fst,
                    gwarp, nwarps, lane);
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tph, 1);
        const unsigned long long c = ldcg(&ctl->qctr[slot]);
        const unsigned F = (unsigned)(c >> 32), T = (unsigned)c;
        // pull when the frontier's (query, edge) relaxations exceed pull_min: the dense rounds
        // in which most active words have most of their queries active (the push pays a
        // red.min per improvement there), not every round with many edge-word steps
        const bool pull = ldcg(&ctl->pcount[slot]) > p.pull_min;  // grid-uniform
        if (gtid == 0) trace_round(p.trace, iters, (long long)T, pull ? 1 : 0);
        if (F == 0) break;
        if (++iters > p.max_iter) {
            if (gtid == 0) atomicOr(flags, C2G_FLAG_ITER_CAP);
            break;
        }
        if (F > p.qcap || ((T + (1u << kBatchTileLog) - 1u) >> kBatchTileLog) > p.mark_cap) {
            if (gtid == 0) atomicOr(flags, C2G_FLAG_BOUNDS);
            break;
        }
        if (gtid == 0) {
            ctl->popped += F;
            ctl->relaxed += T;
        }

        if (p.pull_min != ~0ull) {
            // The previous round's frontier leaves the pull lookup (the lookup of this round,
            // amask[buf], is the one a pull reads; the next round writes amask[buf ^ 1]).
            const unsigned Fp = min((unsigned)(ldcg(&ctl->qctr[(cur + 2) % 3]) >> 32), p.qcap);
            for (unsigned j = gtid; j < Fp; j += nthreads) p.amask[buf ^ 1][ldcg(p.q[buf ^ 1] + j).x] = 0u;
        }
        if (pull) {
            if (gtid == 0) steps += T;
            sbatch_pull(p, buf, &ctl->tilectr[slot], pcs[wib], relax, lane);
        } else {
        // Phase 2: expand.  Warps take tiles of edge-word steps and walk owner runs: the
        // owner's row of distances is read once; its edges are read 32 at a time (one per
        // lane, coalesced) and broadcast by shuffles; each edge costs one 128-byte read of
        // the target's row for the 32 queries of the word, kBatchUnroll rows in flight.
        // Improvements are red.min on the distance and red.or on the target's mask.
        const int2* q = p.q[buf];
        const unsigned* qm = p.qmask[buf];
        const int* mark = p.mark[buf];
        const int tl = batch_tile_log(T, nwarps, p.tile_big_log, p.tile_min_log);
        const unsigned tile = 1u << tl;
        const unsigned ntiles = (T + tile - 1) >> tl;
        unsigned* tctr = &ctl->tilectr[slot];
        unsigned tn = next_tile(tctr, lane);
        for (unsigned t = tn; t < ntiles; t = tn) {
            tn = next_tile(tctr, lane);  // the next tile, fetched while this one runs
            unsigned e0 = t << tl;
            const unsigned e1 = min(e0 + tile, T);
            unsigned o = (unsigned)ldcg(mark + (t << (tl - kBatchTileLog)));
            while (e0 < e1) {
                const unsigned j = o + (unsigned)lane;
                unsigned base = 0x7fffffffu, endv = 0xffffffffu, msk = 0u, rs = 0u;
                int vw = 0;
                bool bad = false;
                if (j < F) {
                    const int2 qe = ldcg(q + j);
                    vw = qe.x;
                    base = (unsigned)qe.y;
                    const int v = vw >> p.logW;
                    rs = (unsigned)__ldg(p.row + v);
                    const unsigned deg = (unsigned)__ldg(p.row + v + 1) - rs;
                    endv = base + deg;
                    bad = rs + deg > p.E || deg == 0u;
                    msk = ldcg(qm + j);
                }
                const unsigned seg_end = min(e1, (unsigned)__shfl_sync(kFull, endv, 31));
                if (__any_sync(kFull, bad) || seg_end <= e0 || o >= F ||
                    (unsigned)__shfl_sync(kFull, (int)base, 0) > e0) {
                    if (lane == 0) atomicOr(flags, C2G_FLAG_BOUNDS);
                    break;
                }
                for (int k = 0; k < 32; ++k) {
                    const unsigned kb = (unsigned)__shfl_sync(kFull, (int)base, k);
                    if (kb >= seg_end) break;
                    const unsigned ke = (unsigned)__shfl_sync(kFull, (int)endv, k);
                    const unsigned lo = max(e0, kb), hi = min(seg_end, ke);
                    if (lo >= hi) continue;
                    const int kvw = __shfl_sync(kFull, vw, k);
                    const unsigned km = (unsigned)__shfl_sync(kFull, (int)msk, k);
                    const unsigned krs = (unsigned)__shfl_sync(kFull, (int)rs, k);
                    const unsigned w = (unsigned)kvw & (unsigned)(W - 1);
                    const unsigned cnt = (unsigned)__popc(km);
                    // slot -> query position of the word's active queries
                    if ((km >> lane) & 1u) qtab[__popc(km & ((1u << lane) - 1u))] = lane;
                    __syncwarp();
                    const int qp = (unsigned)lane < cnt ? qtab[lane] : 0;
                    __syncwarp();
                    int* dw = p.dist + (w << 5);  // + v * Q + query position
                    unsigned* mrow = p.mask + w;  // + (v << logW): mask word of v
                    // L2-coherent: the owner improved in the previous round.
                    const int du = (unsigned)lane < cnt ? ldcg(dw + (size_t)((unsigned)kvw >> p.logW) * Qu + qp) : 0;
                    const unsigned len = hi - lo;
                    const int2* eadj = p.adj + krs + (lo - kb);
                    owner_items<kBatchUnroll>(cnt, len, lane, [&](const int* eis, const int* js) {
                        int2 ew[kBatchUnroll];
                        int dq[kBatchUnroll], qq[kBatchUnroll], cd[kBatchUnroll];
                        bool ok[kBatchUnroll];
#pragma unroll
                        for (int u = 0; u < kBatchUnroll; ++u) {
                            ok[u] = (unsigned)eis[u] < len;
                            ew[u] = ok[u] ? __ldg(eadj + eis[u]) : make_int2(0, 0);
                        }
#pragma unroll
                        for (int u = 0; u < kBatchUnroll; ++u) {
                            dq[u] = __shfl_sync(kFull, du, js[u]);
                            qq[u] = __shfl_sync(kFull, qp, js[u]);
                        }
#pragma unroll
                        for (int u = 0; u < kBatchUnroll; ++u)
                            cd[u] = ok[u] ? ldcg(dw + (size_t)(unsigned)ew[u].x * Qu + qq[u]) : INT_MIN;
#pragma unroll
                        for (int u = 0; u < kBatchUnroll; ++u) {
                            const int nd = dq[u] + ew[u].y;
                            if (nd < cd[u]) {
                                atomicMin(dw + (size_t)(unsigned)ew[u].x * Qu + qq[u], nd);
                                atomicOr(mrow + ((size_t)(unsigned)ew[u].x << p.logW), 1u << qq[u]);
                            }
                        }
                    });
                    if (lane == 0) relax += (long long)cnt * len;
                    steps += len;
                }
                e0 = seg_end;
                o += 32;
            }
        }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tph, 2);
        if (gtid == 0) trace_mid(p.trace, iters - 1);
        ++cur;
        // end of an epoch: the next round's improvements wait in the masks
        if (p.epoch_rounds > 0 && iters >= p.epoch_rounds) break;
    }
    // relax is counted by lane 0 of each warp
    if (lane == 0) {
        atomicAdd((unsigned long long*)&p.counters[0], (unsigned long long)relax);
        atomicAdd((unsigned long long*)&p.counters[1], (unsigned long long)steps);
    }
    if (gtid == 0) {
        ctl->iterations = iters;
        trace_round(p.trace, iters, 0, -1);
    }
}

// Copy dist[V][Q] (first nq queries) into the caller's layout.
__global__ void batch_transpose(const int* __restrict__ dist, int V, int Q, int nq, int* __restrict__ out,
                                int query_major) {
    const size_t total = (size_t)V * (size_t)nq;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        if (query_major) {
            const size_t qi = i / (size_t)V, v = i % (size_t)V;  // coalesced writes
            out[i] = dist[v * Q + qi];
        } else {
            const size_t v = i / (size_t)nq, qi = i % (size_t)nq;
            out[i] = dist[v * Q + qi];
        }
    }
}

// [V][Q] state -> query-major [nq][V] output through a 32 x 32 shared-memory tile: the
// reads cover one 128-byte line of 32 queries per vertex, the writes 32 consecutive
// vertices per query, both coalesced.  (Element-wise, consecutive threads would read with
// a stride of one vertex row.)  Block 32 x 8; grid (V / 32, nq / 32), rounded up.
template <typename S, typename D>
__global__ void __launch_bounds__(256) batch_transpose_qmajor(const S* __restrict__ src, int V, int Q, int nq,
                                                             D* __restrict__ out) {
    __shared__ D tile[32][33];
    const int v0 = (int)blockIdx.x * 32, q0 = (int)blockIdx.y * 32;
    for (int k = (int)threadIdx.y; k < 32; k += 8) {
        const int v = v0 + k, q = q0 + (int)threadIdx.x;
        if (v < V && q < nq) tile[k][threadIdx.x] = (D)src[(size_t)v * (size_t)Q + (size_t)q];
    }
    __syncthreads();
    for (int k = (int)threadIdx.y; k < 32; k += 8) {
        const int q = q0 + k, v = v0 + (int)threadIdx.x;
        if (q < nq && v < V) out[(size_t)q * (size_t)V + (size_t)v] = tile[threadIdx.x][k];
    }
}

// A host output buffer the kernels can write directly: page-locked host memory has a
// device address (over NVLink-C2C on Grace machines), so the results skip the device
// staging copy and the separate device-to-host copy.  nullptr for pageable memory.
static void* mapped_host(void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // clear the error state of the query
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

template <typename S, typename D>
static void launch_transpose_qmajor(const S* src, int V, int Q, int nq, D* out, cudaStream_t st) {
    if (V <= 0 || nq <= 0) return;
    const dim3 grid((unsigned)((V + 31) / 32), (unsigned)((nq + 31) / 32));
    batch_transpose_qmajor<S, D><<<grid, dim3(32, 8), 0, st>>>(src, V, Q, nq, out);
}

// ---------------------------------------------------------------------------------------
// host side

// Blocks of a batched launch: the whole GPU, or the handle's share when several
// batched launches run side by side (the serving loop).
static int grid_blocks(const c2g_graph* g, int per_sm) {
    int b = (int)((float)(per_sm * g->num_sms) * g->grid_scale);
    return b < 1 ? 1 : b;
}

struct BatchWork {
    int* dist = nullptr;
    unsigned* mask = nullptr;
    int2* q[2] = {nullptr, nullptr};
    unsigned* qmask[2] = {nullptr, nullptr};
    int* mark[2] = {nullptr, nullptr};
    TraversalCtl* ctl = nullptr;
    long long* counters = nullptr;
    int* src = nullptr;
    int* seed_off = nullptr;
    int* seed_v = nullptr;
    int* seed_w = nullptr;
    int* stage = nullptr;  // caller-layout copy for host output
    RoundTrace* trace = nullptr;
    unsigned* amask[2] = {nullptr, nullptr};  // pull rounds' lookups of the frontier's lanes
    size_t seed_cap = 0;
    int Q = 0;
    int V = 0;
};

static void batch_free_work(BatchWork* w) {
    if (!w) return;
    void* ptrs[] = {w->dist, w->mask, w->q[0], w->q[1], w->qmask[0], w->qmask[1], w->mark[0], w->mark[1],
                    w->ctl, w->counters, w->src, w->seed_off, w->seed_v, w->seed_w, w->stage, w->trace,
                    w->amask[0], w->amask[1]};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete w;
}

void batch_free(c2g_graph* g) {
    BatchWork* w = reinterpret_cast<BatchWork*>(g->batch);
    if (w && g->last_trace == w->trace) g->last_trace = nullptr;
    batch_free_work(w);
    g->batch = nullptr;
}

static int batch_alloc(c2g_graph* g, int Q, size_t n_seeds) {
    BatchWork* w = reinterpret_cast<BatchWork*>(g->batch);
    if (w && w->Q >= Q && w->seed_cap >= n_seeds) return C2G_OK;
    if (w) batch_free(g);
    w = new BatchWork();
    g->batch = w;
    const size_t V = g->V ? (size_t)g->V : 1;
    const size_t W = (size_t)Q / 32;
    const size_t qcap = V * W;
    const size_t mark_cap = (((size_t)g->E * W) >> kBatchTileLog) + 2;
    C2G_CUDA(cudaMalloc(&w->dist, sizeof(int) * V * (size_t)Q));
    C2G_CUDA(cudaMalloc(&w->mask, sizeof(unsigned) * qcap));
    for (int b = 0; b < 2; ++b) {
        C2G_CUDA(cudaMalloc(&w->q[b], sizeof(int2) * qcap));
        C2G_CUDA(cudaMalloc(&w->qmask[b], sizeof(unsigned) * qcap));
        C2G_CUDA(cudaMalloc(&w->mark[b], sizeof(int) * mark_cap));
    }
    C2G_CUDA(cudaMalloc(&w->ctl, sizeof(TraversalCtl)));
    C2G_CUDA(cudaMalloc(&w->counters, sizeof(long long) * 2));
    C2G_CUDA(cudaMalloc(&w->src, sizeof(int) * (size_t)Q));
    C2G_CUDA(cudaMalloc(&w->seed_off, sizeof(int) * ((size_t)Q + 1)));
    w->seed_cap = n_seeds > 0 ? n_seeds : 1;
    C2G_CUDA(cudaMalloc(&w->seed_v, sizeof(int) * w->seed_cap));
    C2G_CUDA(cudaMalloc(&w->seed_w, sizeof(int) * w->seed_cap));
    C2G_CUDA(cudaMalloc(&w->trace, sizeof(RoundTrace) * (kMaxTraceRounds + 1)));
    for (int b = 0; b < 2; ++b) C2G_CUDA(cudaMalloc(&w->amask[b], sizeof(unsigned) * qcap));
    w->Q = Q;
    w->V = g->V;
    return C2G_OK;
}

// The pull rounds of a batched SSSP launch (p.pull_min: (query, edge) relaxations of the
// frontier above which a round pulls, ~0: never): they need the reverse CSR with int32 weights (a view uses its
// base's, never builds it), whose arrays are set into p here, after they exist.  The pull
// lookups start clear; a launch leaves the entries of its last rounds behind.
static int sssp_pull_setup(c2g_graph* g, BatchWork* w, int Q, BatchParams& p) {
    p.pull_min = ~0ull;
    const float frac = g->sssp_cfg.batch_pull_frac;
    if (!(frac >= 0.f) || g->E == 0) return C2G_OK;
    if (!g->adj_rw) {
        if (g->borrowed) return C2G_OK;
        int rc = build_reverse_int(g);
        if (rc) return rc;
    }
    if (!g->row_r || !g->adj_rw || !g->mark_r) return C2G_OK;
    p.row_r = g->row_r;
    p.adj_rw = g->adj_rw;
    p.mark_r = g->mark_r;
    for (int b = 0; b < 2; ++b)
        C2G_CUDA(cudaMemsetAsync(w->amask[b], 0, sizeof(unsigned) * (size_t)g->V * (size_t)(Q / 32), g->stream));
    p.pull_min = (unsigned long long)((double)frac * (double)g->E * (double)Q);
    return C2G_OK;
}

static void sssp_batch_params(c2g_graph* g, BatchWork* w, int Q, int logW, BatchParams& p) {
    p.row = g->row;
    p.adj = g->adj_w;
    p.E = (unsigned)g->E;
    p.V = g->V;
    p.logW = logW;
    p.Q = Q;
    p.nq = Q;
    p.dist = w->dist;
    p.mask = w->mask;
    for (int b = 0; b < 2; ++b) {
        p.q[b] = w->q[b];
        p.qmask[b] = w->qmask[b];
        p.mark[b] = w->mark[b];
    }
    p.ctl = w->ctl;
    p.sources = w->src;
    p.seed_off = nullptr;
    p.seed_v = w->seed_v;
    p.seed_w = w->seed_w;
    p.qcap = (unsigned)((size_t)g->V * (size_t)(Q / 32));
    p.mark_cap = (unsigned)((((size_t)g->E * (size_t)(Q / 32)) >> kBatchTileLog) + 2);
    p.max_iter = g->sssp_cfg.max_iter;
    p.barrier_ns = g->barrier_ns ? g->barrier_ns : 4000000000ull;
    p.counters = w->counters;
    p.tile_big_log = g->sssp_cfg.batch_tile_big_log;
    p.tile_min_log = g->sssp_cfg.batch_tile_min_log;
    p.epoch_rounds = 0;
    p.trace = w->trace;
    g->last_trace = w->trace;
    p.row_r = nullptr;  // set by sssp_pull_setup when the launch may pull
    p.adj_rw = nullptr;
    p.mark_r = nullptr;
    p.ntiles_r = (unsigned)(((size_t)g->E + (1u << kPullTileLog) - 1) >> kPullTileLog);
    p.pull_min = ~0ull;
    p.amask[0] = w->amask[0];
    p.amask[1] = w->amask[1];
}

static int sssp_batch_results(c2g_graph* g, BatchWork* w, int Q, int32_t nq, int32_t* out, int out_on_device,
                              int query_major, float* ms, long long* counters, TraversalCtl* ctl_out) {
    // Results in the caller's layout (pinned host memory is written directly).
    int* dst = out;
    int* direct = out_on_device ? nullptr : static_cast<int*>(mapped_host(out));
    if (direct) {
        dst = direct;
    } else if (!out_on_device) {
        if (!w->stage) C2G_CUDA(cudaMalloc(&w->stage, sizeof(int) * (size_t)g->V * (size_t)Q));
        dst = w->stage;
    }
    if (query_major)
        launch_transpose_qmajor<int, int>(w->dist, g->V, Q, nq, dst, g->stream);
    else
        batch_transpose<<<g->num_sms * 8, 256, 0, g->stream>>>(w->dist, g->V, Q, nq, dst, query_major);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess && !out_on_device && !direct)
        e = cudaMemcpyAsync(out, dst, sizeof(int) * (size_t)g->V * (size_t)nq, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctl_out, w->ctl, sizeof(TraversalCtl), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counters, w->counters, sizeof(long long) * 2, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    C2G_CUDA(e);
    C2G_CUDA(cudaEventElapsedTime(ms, g->ev0, g->ev1));
    return C2G_OK;
}

int sssp_batch_launch(c2g_graph* g, int32_t nq, const int32_t* sources, const std::vector<int32_t>* seed_off,
                      const std::vector<int32_t>* seed_v, const std::vector<int32_t>* seed_w, int32_t* out,
                      int out_on_device, int query_major, float* ms, long long* counters, TraversalCtl* ctl_out) {
    if (!g->adj_w) return fail(C2G_ERR_UNSUPPORTED, "graph has no int32 weights (wlist)");
    int Q = 32, logW = 0;
    while (Q < nq) {
        Q <<= 1;
        ++logW;
    }
    if ((size_t)g->V * (size_t)(Q / 32) >= (size_t(1) << 31) || (size_t)g->E * (size_t)(Q / 32) >= (size_t(1) << 32))
        return fail(C2G_ERR_RANGE, "batch of %d queries too large for this graph", nq);
    int rc;
    const size_t ns = seed_v ? seed_v->size() : 0;
    if ((rc = batch_alloc(g, Q, ns))) return rc;
    BatchWork* w = reinterpret_cast<BatchWork*>(g->batch);
    int coop = 0, per_sm = 0;
    C2G_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device));
    if (!coop) return fail(C2G_ERR_UNSUPPORTED, "device lacks cooperative launch");
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sssp_batch_persistent, kSsspBatchThreads, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "batch kernel cannot be resident");

    C2G_CUDA(cudaMemcpyAsync(w->src, sources, sizeof(int) * (size_t)nq, cudaMemcpyHostToDevice, g->stream));
    if (seed_off) {
        C2G_CUDA(cudaMemcpyAsync(w->seed_off, seed_off->data(), sizeof(int) * seed_off->size(),
                                 cudaMemcpyHostToDevice, g->stream));
        if (ns) {
            C2G_CUDA(cudaMemcpyAsync(w->seed_v, seed_v->data(), sizeof(int) * ns, cudaMemcpyHostToDevice, g->stream));
            C2G_CUDA(cudaMemcpyAsync(w->seed_w, seed_w->data(), sizeof(int) * ns, cudaMemcpyHostToDevice, g->stream));
        }
    }
    BatchParams p;
    sssp_batch_params(g, w, Q, logW, p);
    if ((rc = sssp_pull_setup(g, w, Q, p))) return rc;
    p.nq = nq;
    p.seed_off = seed_off ? w->seed_off : nullptr;
    C2G_CUDA(cudaMemsetAsync(w->ctl, 0, sizeof(TraversalCtl), g->stream));
    C2G_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(long long) * 2, g->stream));
    void* args[] = {&p};
    C2G_CUDA(cudaEventRecord(g->ev0, g->stream));
    const int blocks = grid_blocks(g, per_sm);
    C2G_CUDA(cudaLaunchCooperativeKernel((const void*)sssp_batch_persistent, dim3(blocks), dim3(kSsspBatchThreads),
                                         args, 0, g->stream));
    C2G_CUDA(cudaEventRecord(g->ev1, g->stream));
    return sssp_batch_results(g, w, Q, nq, out, out_on_device, query_major, ms, counters, ctl_out);
}

// Resident batch (c2g_session): the workspace of Q query slots with every mask clear, and
// one epoch of at most `rounds` rounds from the state the previous epoch left.
int sssp_batch_reserve(c2g_graph* g, int Q, int** dist, unsigned** mask) {
    if (!g->adj_w) return fail(C2G_ERR_UNSUPPORTED, "graph has no int32 weights (wlist)");
    if ((size_t)g->V * (size_t)(Q / 32) >= (size_t(1) << 31) || (size_t)g->E * (size_t)(Q / 32) >= (size_t(1) << 32))
        return fail(C2G_ERR_RANGE, "%d slots too many for this graph", Q);
    int rc;
    if ((rc = batch_alloc(g, Q, 0))) return rc;
    BatchWork* w = reinterpret_cast<BatchWork*>(g->batch);
    C2G_CUDA(cudaMemsetAsync(w->mask, 0, sizeof(unsigned) * (size_t)g->V * (size_t)(Q / 32), g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    *dist = w->dist;
    *mask = w->mask;
    return C2G_OK;
}

int sssp_batch_epoch(c2g_graph* g, int Q, int rounds, float* ms, long long* counters, TraversalCtl* ctl_out) {
    BatchWork* w = reinterpret_cast<BatchWork*>(g->batch);
    if (!w || w->Q < Q) return fail(C2G_ERR_ARG, "resident SSSP batch has no workspace");
    int logW = 0;
    while ((32 << logW) < Q) ++logW;
    int per_sm = 0;
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, sssp_batch_persistent, kSsspBatchThreads, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "batch kernel cannot be resident");
    BatchParams p;
    sssp_batch_params(g, w, Q, logW, p);
    int rc;
    if ((rc = sssp_pull_setup(g, w, Q, p))) return rc;
    p.epoch_rounds = rounds < 1 ? 1 : rounds;
    C2G_CUDA(cudaMemsetAsync(w->ctl, 0, sizeof(TraversalCtl), g->stream));
    C2G_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(long long) * 2, g->stream));
    void* args[] = {&p};
    C2G_CUDA(cudaEventRecord(g->ev0, g->stream));
    C2G_CUDA(cudaLaunchCooperativeKernel((const void*)sssp_batch_persistent, dim3(grid_blocks(g, per_sm)),
                                         dim3(kSsspBatchThreads), args, 0, g->stream));
    C2G_CUDA(cudaEventRecord(g->ev1, g->stream));
    C2G_CUDA(cudaMemcpyAsync(ctl_out, w->ctl, sizeof(TraversalCtl), cudaMemcpyDeviceToHost, g->stream));
    C2G_CUDA(cudaMemcpyAsync(counters, w->counters, sizeof(long long) * 2, cudaMemcpyDeviceToHost, g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    C2G_CUDA(cudaEventElapsedTime(ms, g->ev0, g->ev1));
    return C2G_OK;
}

}  // namespace c2g

// =======================================================================================
// Batched forward push (PPR) with per-query bitmask frontiers.
//
// Same BSP semantics per query as c2g_ppr (src/ppr/purn/Main.cu:149-428): pop r, push
// (1-alpha)*r*w into msg, then res += msg; if res > rmax: pr += alpha*res and activate.
// State is vertex-major [V][Q]: pr float; res, msg and rq (the residual being pushed,
// times 1-alpha) FP64.  A push round marks the target's (vertex, word) touched mask with
// red.or; phase B sweeps the touched masks, applies the messages and activates, building
// the frontier entries (vertex, word) with the activated lanes as their mask.  A round
// with many pushes runs as a pull over the reverse CSR instead (pbatch_pull); both shapes
// produce the same rounds.
namespace c2g {

struct PprBatchParams {
    const int* row;
    const int2* adj;  // (target, float weight bits)
    unsigned E;
    int V;
    int logW, Q, nq;
    float* pr;        // [V][Q]
    double* res;      // [V][Q] FP64 residuals (see ppr.cu: threshold decisions)
    double* msg;      // [V][Q], zero between launches (pull rounds: parts of tile-straddling targets)
    double* rq[2];    // [V][Q] (1-alpha) * residual being pushed, by frontier buffer
    float2* rqf[2];   // the same as a float pair hi + lo (pull rounds)
    unsigned* amask[2];  // [V][W] lanes activated with out-edges, by frontier buffer (pull lookup)
    unsigned* tmask;  // [V][W] touched lanes this round, zero between rounds
    unsigned* slist;  // pull rounds: the (vertex, word)s a pull left in tmask (tile-straddling targets)
    unsigned slist_cap;
    unsigned* dmask;  // [V][W] lanes activated without out-edges (popped next round), zero between launches
    int2* q[2];       // frontier entries (v*W + w, edge base)
    unsigned* qmask[2];
    int* mark[2];
    int2* dangle;     // (v*W + w, lanes) activated without out-edges, popped next round
    TraversalCtl* ctl;
    const int* sources;
    const int* seed_off;  // seeded mode: per-query record offsets
    const int* seed_v;
    const float* seed_w;
    float alpha, rmax, r0, pr0;
    int seeded;
    int max_iter;
    unsigned qcap, mark_cap;
    unsigned long long barrier_ns;
    long long* counters;  // [2] pushes (query, edge), edge-word steps
    // pull rounds: reverse CSR (source, weight bits) with tile owners; a round pulls when
    // its pushes exceed pull_min
    const int* row_r;
    const int2* adj_r;
    const int* mark_r;
    unsigned ntiles_r;
    unsigned long long pull_min;
    int epoch_rounds;  // > 0: an epoch of a resident batch (state at rest in the arrays; at most this many rounds)
    int cur0;          // round index the epoch starts at (its parity picks the frontier buffers)
    RoundTrace* trace;  // [kMaxTraceRounds + 1] per-round trace
};

__device__ __forceinline__ FrontierOut pbatch_out(const PprBatchParams& p, int buf, int slot) {
    FrontierOut o;
    o.q = p.q[buf];
    o.val = reinterpret_cast<float*>(p.qmask[buf]);  // mask bits travel in the value slot
    o.mark = p.mark[buf];
    o.ctr = &p.ctl->qctr[slot];
    o.cap = p.qcap;
    o.mark_cap = p.mark_cap;
    o.log_tile = kBatchTileLog;
    o.flags = &p.ctl->flags;
    return o;
}

// Launch shape of the batched PPR: 2 blocks of 512 threads per SM (64 registers).  With the
// pull rounds staged through shared memory it beats 3 x 384 (56 registers) by about 1% at
// 256 sources, scale 22 (766 vs 775 ms: faster pulls, slower pushes) and 4 x 256 (778 ms);
// before the staging 3 x 384 had been the faster one (962 vs 1,030 ms).
constexpr int kPprBatchThreads = 512;
constexpr int kPprBatchBlocksPerSm = 2;
constexpr int kPprBatchUnroll = 3;  // push items in flight per lane

// Apply of one (vertex, word) to the lanes that received messages: res += m; a lane whose
// residual exceeds rmax adds alpha * res to pr and activates.  An activated lane with
// out-edges stores (1-alpha) * res as the residual it pushes next round (in rq[ob]) and
// zeroes res; one without out-edges keeps res until the next round pops it.  The word's
// activated lanes go to the next frontier (and to amask[ob], the pull rounds' lookup),
// or to the dangling list.  force = true: the seeded first hop (activate every touched
// lane, no messages).  psum (lane 0) accumulates the next round's pushes.
__device__ __forceinline__ void pbatch_apply_word(const PprBatchParams& p, bool force, int ob, int vw, int dg,
                                                  size_t off, bool mine, double r, double m, float pv,
                                                  unsigned long long rmax_bits, WarpStage& fst, const FrontierOut& out,
                                                  unsigned* dctr, unsigned long long& psum, int lane) {
    bool act = false;
    if (mine) {
        double rr = r;
        if (!force) rr += m;
        // rr and rmax are non-negative: compare their bit patterns
        if (force || c2g_dbits(rr) > rmax_bits) {
            if (!force) p.pr[off] = pv + (float)((double)p.alpha * rr);
            act = true;
            if (dg > 0) {
                const double q = (1.0 - (double)p.alpha) * rr;  // (1-alpha)*r_u (src/ppr/purn/Main.cu:288)
                p.rq[ob][off] = q;
                if (c2g_split_ok(q)) {  // float pair for pull rounds (fp64_mul.h)
                    const c2g_pair hl = c2g_split_pair(q);
                    p.rqf[ob][off] = make_float2(c2g_bitsf(hl.hi), c2g_bitsf(hl.lo));
                } else {
                    const float hi = __double2float_rz(q);
                    p.rqf[ob][off] = make_float2(hi, __double2float_rz(q - (double)hi));
                }
                p.res[off] = 0.0;
            } else {
                p.res[off] = rr;  // popped (zeroed) at the top of the next round
            }
        } else {
            p.res[off] = rr;
        }
    }
    const unsigned bits = __ballot_sync(kFull, act);
    if (bits && lane == 0) {
        if (dg == 0) {
            const unsigned slot = atomicAdd(dctr, 1u);
            if (slot < p.qcap)
                p.dangle[slot] = make_int2(vw, (int)bits);
            else
                atomicOr(&p.ctl->flags, C2G_FLAG_QUEUE_OVERFLOW);
            p.dmask[vw] = bits;  // the same lanes at rest, for an epoch boundary
        } else {
            p.amask[ob][vw] = bits;
            psum += (unsigned long long)__popc(bits) * (unsigned long long)dg;
        }
    }
    stage_push(fst, out, lane == 0 && bits != 0u && dg > 0, vw, dg, __int_as_float((int)bits));
}

// Apply sweep: every (vertex, word) whose touched mask is non-zero applies its messages
// lane by lane (lane = query) and activates; the mask is cleared.  Pushes mark targets with
// red.or, so the push never waits on an atomic's return; the sweep reads V * W mask words
// per round.  After a pull round only the targets whose in-edges cross a tile boundary
// are left, and the sweep visits just those, from the list the pull wrote (list != null:
// nlist word indices; 842 vs 875 ms per 256-query batch at scale 22 against sweeping all
// V * W words).  A warp takes 32 words at a time (their degrees loaded lane-parallel) and
// applies up to kApplyGroup touched words at once: all their residual, message and pr
// loads are issued before any of them is used, so the words' memory latencies overlap
// instead of adding up.  (Loading 2 or 4 blocks of 32 mask words before applying any
// measured slower: 852 and 870 ms.)
constexpr int kApplyGroup = 3;  // 4 spills at 64 registers

__device__ __forceinline__ unsigned pbatch_sweep(const PprBatchParams& p, bool force, int ob, const unsigned* list,
                                                 unsigned nlist, WarpStage& fst, const FrontierOut& out,
                                                 unsigned* dctr, unsigned long long& psum, unsigned gwarp,
                                                 unsigned nwarps, int lane) {
    const unsigned nm = list ? nlist : (unsigned)p.V << p.logW;
    const unsigned long long rmax_bits = c2g_dbits((double)p.rmax);
    unsigned cnt = 0;
    for (unsigned b = gwarp * 32u; b < nm; b += nwarps * 32u) {
        const unsigned pos = b + (unsigned)lane;
        const unsigned i = pos < nm ? (list ? ldcg(list + pos) : pos) : 0u;  // this lane's (vertex, word)
        const unsigned tm = pos < nm ? ldcg(p.tmask + i) : 0u;
        int dg = 0;
        if (tm) {
            p.tmask[i] = 0u;
            const int v = (int)(i >> p.logW);
            dg = __ldg(p.row + v + 1) - __ldg(p.row + v);
        }
        unsigned nz = __ballot_sync(kFull, tm != 0u);
        cnt += (unsigned)__popc(tm);  // touched (vertex, query) lanes seen by this lane
        while (nz) {
            int ks[kApplyGroup];
#pragma unroll
            for (int u = 0; u < kApplyGroup; ++u) {
                ks[u] = nz ? __ffs(nz) - 1 : -1;
                nz &= nz - 1u;
            }
            // element (v, w*32 + lane) of a [V][Q] array sits at (v*W + w)*32 + lane
            double r[kApplyGroup], m[kApplyGroup];
            float pv[kApplyGroup];
#pragma unroll
            for (int u = 0; u < kApplyGroup; ++u) {
                const int k = ks[u] < 0 ? 0 : ks[u];
                const unsigned ln = ks[u] < 0 ? 0u : (unsigned)__shfl_sync(kFull, (int)tm, k);
                const unsigned vw = (unsigned)__shfl_sync(kFull, (int)i, k);
                const size_t off = ((size_t)vw << 5) + lane;
                const bool mine = (ln >> lane) & 1u;
                r[u] = mine ? ldcg(p.res + off) : 0.0;
                m[u] = (mine && !force) ? ldcg(p.msg + off) : 0.0;
                pv[u] = (mine && !force) ? ldcg(p.pr + off) : 0.f;
            }
#pragma unroll
            for (int u = 0; u < kApplyGroup; ++u) {
                if (ks[u] < 0) break;  // warp-uniform
                const unsigned ln = (unsigned)__shfl_sync(kFull, (int)tm, ks[u]);
                const int dgu = __shfl_sync(kFull, dg, ks[u]);
                const int vw = __shfl_sync(kFull, (int)i, ks[u]);
                const size_t off = ((size_t)(unsigned)vw << 5) + lane;
                const bool mine = (ln >> lane) & 1u;
                if (mine && !force) p.msg[off] = 0.0;
                pbatch_apply_word(p, force, ob, vw, dgu, off, mine, r[u], m[u], pv[u], rmax_bits, fst, out, dctr,
                                  psum, lane);
            }
        }
    }
    stage_flush(fst, out);
    return cnt;
}

// ---------------------------------------------------------------------------------------
// Pull round.  In the dense middle of a batch most (vertex, query) pairs are active, and a
// push does one FP64 read-modify-write per (edge, query) on a message array far larger
// than L2.  A pull round instead walks the reverse CSR: for each target v and query word,
// the warp reads v's in-edges (u, w(u,v)), looks up u's active lanes (amask) and gathers
// the pushed residuals of those lanes (one coalesced 256-byte row segment per edge and
// word), summing the messages rq * w in registers.  The sums are float pairs hi + lo
// (about 47 bits of relative precision): the product is hi*w + lo*w with its rounding
// error recovered by an FMA, and each add is an error-free two-sum whose error joins lo.
// Relative precision matters here, not absolute: a message sum decides res > rmax at the
// scale of rmax, far below the largest sums.  A target whose in-edges lie in one tile is
// applied by the warp that summed them; only targets whose in-edges cross a tile boundary
// add their parts to msg (FP64 atomics) for the apply sweep that follows, as after a push.
// In-edges are cut into tiles of 2^kPullTileLog; warps take (tile, word group) items from
// the round's queue, kPullWords query words per item.
constexpr int kPullWords = 4;  // query words per pull item
constexpr int kPullEdges = 2;  // in-edges whose rq rows are gathered before they are summed

// Owner v's message sums of the item's words are complete (hi + lo per lane).  An owner
// whose in-edges lie in this tile has them all: it is applied here, by the pulling warp
// (the pullers read the other round parity's rq pairs and activity masks, so this apply
// does not disturb them).  An owner whose in-edges cross a tile boundary adds its part to
// msg in FP64 (atomics) and marks tmask; the apply after the barrier finishes it.  The
// first part to mark a (vertex, word) appends it to slist (counter sctr), so that apply
// visits only the listed words instead of sweeping all V * W (at most one owner straddles
// each tile boundary, so the list holds at most ntiles_r * W words).
__device__ __forceinline__ unsigned pbatch_pull_owner(const PprBatchParams& p, int v, unsigned w0, bool whole,
                                                      const float (&sh)[kPullWords], const float (&sl)[kPullWords],
                                                      int ob, unsigned long long rmax_bits, WarpStage& fst,
                                                      const FrontierOut& out, unsigned* dctr, unsigned* sctr,
                                                      unsigned long long& psum, int lane) {
    const unsigned W = 1u << p.logW;
    unsigned cnt = 0;
    if (!whole) {
#pragma unroll
        for (int j = 0; j < kPullWords; ++j) {
            if (w0 + j >= W) break;  // warp-uniform
            const bool nz = sh[j] != 0.f;
            const unsigned bits = __ballot_sync(kFull, nz);
            if (bits) {
                const size_t vw = ((size_t)(unsigned)v << p.logW) + w0 + j;
                if (nz)
                    atomicAdd(p.msg + (vw << 5) + lane, c2g_float_bits_to_double(__float_as_uint(sh[j])) +
                                                            c2g_float_bits_to_double(__float_as_uint(sl[j])));
                if (lane == 0 && atomicOr(p.tmask + vw, bits) == 0u) {
                    const unsigned k = atomicAdd(sctr, 1u);
                    if (k < p.slist_cap) p.slist[k] = (unsigned)vw;
                }
            }
        }
        return 0;
    }
    const int dg = __ldg(p.row + v + 1) - __ldg(p.row + v);
    double r[kPullWords];
    float pv[kPullWords];
#pragma unroll
    for (int j = 0; j < kPullWords; ++j) {
        const size_t off = (size_t)v * (size_t)p.Q + ((w0 + j) << 5) + lane;
        const bool nz = sh[j] != 0.f;
        r[j] = nz ? ldcg(p.res + off) : 0.0;
        pv[j] = nz ? ldcg(p.pr + off) : 0.f;
    }
#pragma unroll
    for (int j = 0; j < kPullWords; ++j) {
        if (w0 + j >= W) break;  // warp-uniform
        const bool nz = sh[j] != 0.f;
        if (!__any_sync(kFull, nz)) continue;
        cnt += nz ? 1u : 0u;
        const size_t off = (size_t)v * (size_t)p.Q + ((w0 + j) << 5) + lane;
        const double m = c2g_float_bits_to_double(__float_as_uint(sh[j])) +
                         c2g_float_bits_to_double(__float_as_uint(sl[j]));
        pbatch_apply_word(p, false, ob, (int)(((unsigned)v << p.logW) + w0 + j), dg, off, nz, r[j], m, pv[j],
                          rmax_bits, fst, out, dctr, psum, lane);
    }
    return cnt;
}

// Phase A of a pull round.  A warp takes (tile, word group) items from the round's queue
// and walks the tile's owners one by one: for each owner, its in-edges in the tile in
// chunks of 32 (loaded lane-parallel and staged in pc), the pushed residuals of
// kPullEdges in-edges gathered before they are summed, two query words per packed
// instruction (f32x2.h).
__device__ __forceinline__ unsigned pbatch_pull(const PprBatchParams& p, int buf, int ob, unsigned* qctr,
                                                PullChunk& pc, WarpStage& fst, const FrontierOut& out, unsigned* dctr,
                                                unsigned* sctr, unsigned long long& psum, int lane, bool& bad) {
    const unsigned W = 1u << p.logW;
    const int lg = p.logW >= 2 ? p.logW - 2 : 0;  // word groups per tile = 2^lg (kPullWords = 4)
    const unsigned nitems = p.ntiles_r << lg;
    const unsigned* am = p.amask[buf];
    const float2* rqb = p.rqf[buf];
    const unsigned tw = 1u << kPullTileLog;
    const unsigned long long rmax_bits = c2g_dbits((double)p.rmax);
    unsigned cnt = 0;
    unsigned itn = next_tile(qctr, lane);
    for (unsigned it = itn; it < nitems; it = itn) {
        itn = next_tile(qctr, lane);  // the next item, fetched while this one runs
        // word group major: all tiles of one word group, then the next, so the residual
        // rows that L2 holds for the busiest sources are one word group's (1 KB per source,
        // not 2 at 256 queries): 818 vs 843 ms per 256-query batch at scale 22
        const unsigned t = it % p.ntiles_r;
        const unsigned w0 = (it / p.ntiles_r) * (unsigned)kPullWords;
        const unsigned e0 = t << kPullTileLog;
        const unsigned e1 = min(e0 + tw, p.E);
        int v = __ldg(p.mark_r + t);  // owner of in-edge e0
        unsigned vs = (unsigned)__ldg(p.row_r + v);
        for (;;) {
            const unsigned ve = (unsigned)__ldg(p.row_r + v + 1);
            const unsigned ea = max(vs, e0), ez = min(ve, e1);
            if (ea < ez) {  // warp-uniform: v has in-edges in this tile
                // message sums hi + lo of words (0, 1) and (2, 3), packed
                f32x2 sh2[kPullWords / 2], sl2[kPullWords / 2];
#pragma unroll
                for (int j = 0; j < kPullWords / 2; ++j) sh2[j] = sl2[j] = 0ull;
                for (unsigned b = ea; b < ez; b += 32u) {
                    const unsigned e = b + (unsigned)lane;
                    int src = 0;
                    float wt = 0.f;
                    unsigned mk[kPullWords];
#pragma unroll
                    for (int j = 0; j < kPullWords; ++j) mk[j] = 0u;
                    if (e < ez) {
                        const int2 ed = __ldg(p.adj_r + e);
                        if ((unsigned)ed.x >= (unsigned)p.V) {
                            bad = true;
                        } else if (ed.y > 0) {  // positive weights only, as the push
                            src = ed.x;
                            wt = __int_as_float(ed.y);
                            const unsigned* ms = am + ((size_t)(unsigned)src << p.logW) + w0;
                            if (W >= 4u) {  // four words, 16-byte aligned
                                const uint4 m4 = ldcg(reinterpret_cast<const uint4*>(ms));
                                mk[0] = m4.x;
                                mk[1] = m4.y;
                                mk[2] = m4.z;
                                mk[3] = m4.w;
                            } else {
#pragma unroll
                                for (int j = 0; j < kPullWords; ++j)
                                    if ((unsigned)j < W) mk[j] = ldcg(ms + j);
                            }
                        }
                    }
                    // only in-edges whose source has an active lane in the item's words are
                    // staged (in order): the others would add exact zeros
                    const bool live = (mk[0] | mk[1] | mk[2] | mk[3]) != 0u;
                    const unsigned lm = __ballot_sync(kFull, live);
                    const unsigned n = (unsigned)__popc(lm);
                    __syncwarp();  // the previous chunk's reads are done
                    if (live) {
                        const unsigned at = (unsigned)__popc(lm & ((1u << lane) - 1u));
                        pc.ed[at] = make_int2(src, __float_as_int(wt));
                        pc.mk[at] = make_uint4(mk[0], mk[1], mk[2], mk[3]);
                    }
                    __syncwarp();
                    for (unsigned k0 = 0; k0 < n; k0 += kPullEdges) {
                        // gather the pushed residuals of kPullEdges in-edges, then add them
                        float2 qb[kPullEdges][kPullWords];
                        float wk[kPullEdges];
#pragma unroll
                        for (int h = 0; h < kPullEdges; ++h) {
                            const unsigned k = k0 + h < n ? k0 + h : n - 1u;
                            const int2 ek = pc.ed[k];
                            const uint4 mq = pc.mk[k];
                            wk[h] = __int_as_float(ek.y);
                            const int u = ek.x;
#pragma unroll
                            for (int j = 0; j < kPullWords; ++j) {
                                const unsigned mj = j == 0 ? mq.x : j == 1 ? mq.y : j == 2 ? mq.z : mq.w;
                                const bool on = k0 + h < n && ((mj >> lane) & 1u);
                                qb[h][j] = on ? ldcg(rqb + ((size_t)(unsigned)u << (p.logW + 5)) + ((w0 + j) << 5) +
                                                     lane)
                                              : make_float2(0.f, 0.f);
                            }
                        }
#pragma unroll
                        for (int h = 0; h < kPullEdges; ++h) {
                            const f32x2 w2 = f2_pack(wk[h], wk[h]);
                            const f32x2 nw2 = f2_pack(-wk[h], -wk[h]);
#pragma unroll
                            for (int j = 0; j < kPullWords / 2; ++j) {
                                // message (hi + lo) * w = pm + pe; two-sum of sh + pm, for words
                                // 2j and 2j+1 at once.  npm = -pm exactly (round-to-nearest is
                                // symmetric), so every line rounds as the scalar form
                                //   pm = hi*w, pe = fma(lo, w, fma(hi, w, -pm)), s = sh + pm,
                                //   bv = s - sh, av = s - bv, te = (sh - av) + (pm - bv),
                                //   sl += te + pe, sh = s
                                // does: pm - bv = -(npm + bv).
                                const f32x2 hi = f2_pack(qb[h][2 * j].x, qb[h][2 * j + 1].x);
                                const f32x2 lo = f2_pack(qb[h][2 * j].y, qb[h][2 * j + 1].y);
                                const f32x2 npm = f2_mul(hi, nw2);
                                const f32x2 pe = f2_fma(lo, w2, f2_fma(hi, w2, npm));
                                const f32x2 s2 = f2_sub(sh2[j], npm);
                                const f32x2 bv = f2_sub(s2, sh2[j]);
                                const f32x2 av = f2_sub(s2, bv);
                                const f32x2 te = f2_sub(f2_sub(sh2[j], av), f2_add(npm, bv));
                                sl2[j] = f2_add(sl2[j], f2_add(te, pe));
                                sh2[j] = s2;
                            }
                        }
                    }
                }
                float sh[kPullWords], sl[kPullWords];
#pragma unroll
                for (int j = 0; j < kPullWords / 2; ++j) {
                    f2_unpack(sh2[j], sh[2 * j], sh[2 * j + 1]);
                    f2_unpack(sl2[j], sl[2 * j], sl[2 * j + 1]);
                }
                cnt += pbatch_pull_owner(p, v, w0, vs >= e0 && ve <= e1, sh, sl, ob, rmax_bits, fst, out, dctr,
                                         sctr, psum, lane);
            }
            if (ve >= e1) break;
            ++v;
            vs = ve;
        }
    }
    stage_flush(fst, out);
    return cnt;
}

// Start of an epoch of a resident batch: round `slot`'s frontier from the state at rest,
// the activity masks of buffer b (lanes activated with out-edges, their pushed residuals
// in rq[b] / rqf[b]) and dmask (lanes activated without out-edges), as the apply sweep
// of the previous round would have built it: entries (vertex, word) with their lanes,
// the dangling list, and the round's push count.
__device__ __noinline__ void pbatch_rebuild(const PprBatchParams& p, int b, int slot, WarpStage& fst,
                                               unsigned gwarp, unsigned nwarps, int lane) {
    const unsigned nm = (unsigned)p.V << p.logW;
    const FrontierOut out = pbatch_out(p, b, slot);
    unsigned long long ps = 0;
    for (unsigned base = gwarp * 32u; base < nm; base += nwarps * 32u) {
        const unsigned i = base + (unsigned)lane;
        unsigned a = 0u, d = 0u;
        int deg = 0;
        if (i < nm) {
            a = ldcg(p.amask[b] + i);
            d = ldcg(p.dmask + i);
            if (a) {
                const int v = (int)(i >> p.logW);
                deg = __ldg(p.row + v + 1) - __ldg(p.row + v);
            }
        }
        if (a && deg > 0) ps += (unsigned long long)__popc(a) * (unsigned long long)deg;
        stage_push(fst, out, a != 0u && deg > 0, (int)i, deg, __int_as_float((int)a));
        if (d) {
            const unsigned k = atomicAdd(&p.ctl->dctr[slot], 1u);
            if (k < p.qcap)
                p.dangle[k] = make_int2((int)i, (int)d);
            else
                atomicOr(&p.ctl->flags, C2G_FLAG_QUEUE_OVERFLOW);
        }
    }
    stage_flush(fst, out);
    for (int o = 16; o >= 1; o >>= 1) ps += __shfl_xor_sync(kFull, ps, o);
    if (lane == 0 && ps) atomicAdd(&p.ctl->pcount[slot], ps);
}

__global__ void __launch_bounds__(kPprBatchThreads, kPprBatchBlocksPerSm)
    ppr_batch_persistent(const PprBatchParams p) {
    TraversalCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nthreads = gridDim.x * blockDim.x;
    const unsigned gwarp = gtid >> 5, nwarps = nthreads >> 5;
    const int W = 1 << p.logW;
    const unsigned Qu = (unsigned)p.Q;
    __shared__ StageSmem sm;
    const int wib = threadIdx.x >> 5;
    WarpStage fst{sm.v0[wib], sm.d0[wib], sm.x0[wib], 0};
    int* qtab = sm.v1[wib];  // slot -> query position table of the owner being expanded
    __shared__ PullChunk pcs[kPprBatchThreads / 32];  // pull rounds' in-edge chunks
    const double one_m_a = 1.0 - (double)p.alpha;
    unsigned long long tph = globaltimer_ns();
    unsigned long long psum = 0;  // next round's pushes counted by this warp (lane 0)

    if (p.epoch_rounds == 0) {
    // Init: pr = res = 0 (msg, tmask, amask and dmask are zero between launches).
    {
        const size_t n4 = ((size_t)p.V * (size_t)p.Q) >> 2;
        float4* a4 = reinterpret_cast<float4*>(p.pr);
        double2* b2 = reinterpret_cast<double2*>(p.res);
        const float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        const double2 zd = make_double2(0.0, 0.0);
        for (size_t i = gtid; i < n4; i += nthreads) {
            a4[i] = z;
            b2[2 * i] = zd;
            b2[2 * i + 1] = zd;
        }
    }
    if (!grid_sync(bar, flags, p.barrier_ns)) return;
    // Sources: base mode puts r0 on the source; seeded mode applies the host-side first
    // hop (records + kept out-edges) to pr/res, a warp per query with its lanes over the
    // records and edges (a hub source has thousands).  Either way the touched lanes are
    // marked.
    for (unsigned qi = gwarp; qi < (unsigned)p.nq; qi += nwarps) {
        const int s = p.sources[qi];
        const int w = (int)(qi >> 5);
        const unsigned bit = 1u << (qi & 31);
        if (!p.seeded) {
            if (lane == 0) {
                atomicAdd(p.pr + (size_t)s * p.Q + qi, p.pr0);
                atomicAdd(p.res + (size_t)s * p.Q + qi, (double)p.r0);
                atomicOr(p.tmask + ((size_t)s << p.logW) + w, bit);
            }
        } else {
            if (lane == 0) atomicAdd(p.pr + (size_t)s * p.Q + qi, p.alpha);
            const int rs = __ldg(p.row + s), re = __ldg(p.row + s + 1);
            const int n_rec = p.seed_off[qi + 1] - p.seed_off[qi];
            for (int k = lane; k < n_rec + (re - rs); k += 32) {
                int v;
                float wt;
                if (k < n_rec) {
                    v = p.seed_v[p.seed_off[qi] + k];
                    wt = p.seed_w[p.seed_off[qi] + k];
                } else {
                    const int2 ew = __ldg(p.adj + rs + (k - n_rec));
                    v = ew.x;
                    wt = __int_as_float(ew.y);
                }
                atomicAdd(p.pr + (size_t)v * p.Q + qi, (float)(one_m_a * (double)p.alpha * (double)wt));
                atomicAdd(p.res + (size_t)v * p.Q + qi, one_m_a * (double)wt);
                atomicOr(p.tmask + ((size_t)v << p.logW) + w, bit);
            }
        }
    }
    if (!grid_sync(bar, flags, p.barrier_ns)) return;
    // Round-1 frontier: every touched (vertex, word) activates its touched lanes.
    pbatch_sweep(p, true, 1, nullptr, 0u, fst, pbatch_out(p, 1, 1), &ctl->dctr[1], psum, gwarp, nwarps, lane);
    if (lane == 0 && psum) atomicAdd(&ctl->pcount[1], psum);
    psum = 0;
    if (!grid_sync(bar, flags, p.barrier_ns)) return;
    } else {
        // An epoch of a resident batch: the state is at rest in the arrays.
        pbatch_rebuild(p, p.cur0 & 1, p.cur0 % 3, fst, gwarp, nwarps, lane);
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
    }
    phase_mark(ctl->phase_ns, tph, 0);

    long long pushes = 0, steps = 0;
    unsigned long long touched = 0;
    int cur = p.epoch_rounds > 0 ? p.cur0 : 1, iters = 0;
    bool bad = false;
    for (;;) {
        const unsigned long long c = ldcg(&ctl->qctr[cur % 3]);
        const unsigned F = (unsigned)(c >> 32), T = (unsigned)c;
        const unsigned D = min(ldcg(&ctl->dctr[cur % 3]), p.qcap);
        const unsigned long long P = ldcg(&ctl->pcount[cur % 3]);  // this round's (query, edge) pushes
        const int buf = cur & 1, ob = (cur + 1) & 1;
        if (gtid == 0) trace_round(p.trace, iters, (long long)P, P > p.pull_min ? 1 : 0);
        if (F == 0 && D == 0) break;
        // end of an epoch: the state rests in the arrays for the next one
        if (p.epoch_rounds > 0 && iters >= p.epoch_rounds) break;
        if (++iters > p.max_iter) {
            // Round cap: activated lanes keep their residual (never popped); their
            // activity masks are cleared for the next launch.
            if (gtid == 0) atomicOr(flags, C2G_FLAG_ITER_CAP);
            for (unsigned j = gwarp; j < F; j += nwarps) {
                const int vw = ldcg(p.q[buf] + j).x;
                const unsigned lanes = ldcg(p.qmask[buf] + j);
                const size_t off = (size_t)(vw >> p.logW) * p.Q + ((vw & (W - 1)) << 5) + lane;
                if ((lanes >> lane) & 1u) p.res[off] = ldcg(p.rq[buf] + off) / one_m_a;
                if (lane == 0) p.amask[buf][vw] = 0u;
            }
            for (unsigned j = gwarp; j < D; j += nwarps)
                if (lane == 0) p.dmask[ldcg(p.dangle + j).x] = 0u;
            break;
        }
        // Pop the activated lanes without out-edges.
        for (unsigned j = gwarp; j < D; j += nwarps) {
            const int2 dv = ldcg(p.dangle + j);
            const size_t off = (size_t)(dv.x >> p.logW) * p.Q + ((dv.x & (W - 1)) << 5) + lane;
            if (((unsigned)dv.y >> lane) & 1u) p.res[off] = 0.0;
            if (lane == 0) p.dmask[dv.x] = 0u;
        }
        if (F == 0) break;
        const bool pull = P > p.pull_min;  // grid-uniform
        // A pull round applies targets while it pulls: the pops above (residuals) and the
        // dangling list they read (which the applies refill) must be done first.
        if (pull && D > 0 && !grid_sync(bar, flags, p.barrier_ns)) return;
        if (F > p.qcap || ((T + (1u << kBatchTileLog) - 1u) >> kBatchTileLog) > p.mark_cap) {
            if (gtid == 0) atomicOr(flags, C2G_FLAG_BOUNDS);
            break;
        }
        const int nslot = (cur + 1) % 3, fslot = (cur + 2) % 3;
        if (gtid == 0) {
            ctl->qctr[fslot] = 0ull;
            ctl->dctr[fslot] = 0u;
            ctl->tilectr[fslot] = 0u;
            ctl->listctr[fslot] = 0u;
            ctl->pcount[fslot] = 0ull;
            ctl->popped += F;
            ctl->relaxed += T;
        }
        if (pull) {
            // Pull round, phase A: gather and sum the messages per target, and apply the
            // targets whose in-edges lie in one tile.
            if (gtid == 0) {
                pushes += (long long)P;
                steps += T;
            }
            touched += pbatch_pull(p, buf, ob, &ctl->tilectr[cur % 3], pcs[wib], fst, pbatch_out(p, ob, nslot),
                                   &ctl->dctr[nslot], &ctl->listctr[cur % 3], psum, lane, bad);
        } else {
            // Push round, phase A: push along the frontier's edges (owner runs, as in the
            // SSSP batch): red.add of the FP64 message per active lane, red.or of the
            // word's sending lanes into the target's touched mask.
            const int2* q = p.q[buf];
            const unsigned* qm = p.qmask[buf];
            const int* mark = p.mark[buf];
            const double* rqb = p.rq[buf];
            const int tl = batch_tile_log(T, nwarps, kPushTileBig, kPushTileMin);
            const unsigned tile = 1u << tl;
            const unsigned ntiles = (T + tile - 1) >> tl;
            unsigned* tctr = &ctl->tilectr[cur % 3];
            unsigned tn = next_tile(tctr, lane);
            for (unsigned t = tn; t < ntiles; t = tn) {
                tn = next_tile(tctr, lane);  // the next tile, fetched while this one runs
                unsigned e0 = t << tl;
                const unsigned e1 = min(e0 + tile, T);
                unsigned o = (unsigned)ldcg(mark + (t << (tl - kBatchTileLog)));
                while (e0 < e1) {
                    const unsigned j = o + (unsigned)lane;
                    unsigned base = 0x7fffffffu, endv = 0xffffffffu, msk = 0u, rs = 0u;
                    int vw = 0;
                    bool badj = false;
                    if (j < F) {
                        const int2 qe = ldcg(q + j);
                        vw = qe.x;
                        base = (unsigned)qe.y;
                        const int v = vw >> p.logW;
                        rs = (unsigned)__ldg(p.row + v);
                        const unsigned deg = (unsigned)__ldg(p.row + v + 1) - rs;
                        endv = base + deg;
                        badj = rs + deg > p.E || deg == 0u;
                        msk = ldcg(qm + j);
                    }
                    const unsigned seg_end = min(e1, (unsigned)__shfl_sync(kFull, endv, 31));
                    if (__any_sync(kFull, badj) || seg_end <= e0 || o >= F ||
                        (unsigned)__shfl_sync(kFull, (int)base, 0) > e0) {
                        if (lane == 0) atomicOr(flags, C2G_FLAG_BOUNDS);
                        break;
                    }
                    for (int k = 0; k < 32; ++k) {
                        const unsigned kb = (unsigned)__shfl_sync(kFull, (int)base, k);
                        if (kb >= seg_end) break;
                        const unsigned ke = (unsigned)__shfl_sync(kFull, (int)endv, k);
                        const unsigned lo = max(e0, kb), hi = min(seg_end, ke);
                        if (lo >= hi) continue;
                        const int kvw = __shfl_sync(kFull, vw, k);
                        const unsigned km = (unsigned)__shfl_sync(kFull, (int)msk, k);
                        const unsigned krs = (unsigned)__shfl_sync(kFull, (int)rs, k);
                        const unsigned w = (unsigned)kvw & (unsigned)(W - 1);
                        const unsigned cnt = (unsigned)__popc(km);
                        // slot -> query position of the word's active queries
                        if ((km >> lane) & 1u) qtab[__popc(km & ((1u << lane) - 1u))] = lane;
                        __syncwarp();
                        const int qp = (unsigned)lane < cnt ? qtab[lane] : 0;
                        __syncwarp();
                        double* mw = p.msg + (w << 5);  // + v * Q + query position
                        unsigned* trow = p.tmask + w;   // + (v << logW): touched word of v
                        // (1-alpha)*r_u of slot `lane`'s query, stored by the apply that
                        // activated it (src/ppr/purn/Main.cu:288)
                        const double qu = (unsigned)lane < cnt
                                              ? ldcg(rqb + (size_t)((unsigned)kvw >> p.logW) * Qu + (w << 5) + qp)
                                              : 0.0;
                        const DSplit qs = c2g_dsplit(qu);
                        // exponent and high significand in one word (0: residual outside the
                        // integer product's range, multiply on the FP64 pipe)
                        const unsigned qpk = c2g_mul_q_ok(qs) ? ((unsigned)qs.e << 21) | qs.hi : 0u;
                        const unsigned len = hi - lo;
                        const int2* eadj = p.adj + krs + (lo - kb);
                        owner_items<kPprBatchUnroll>(cnt, len, lane, [&](const int* eis, const int* js) {
                            int2 ew[kPprBatchUnroll];
                            bool ok[kPprBatchUnroll];
#pragma unroll
                            for (int u = 0; u < kPprBatchUnroll; ++u) {
                                ok[u] = (unsigned)eis[u] < len;
                                ew[u] = ok[u] ? __ldg(eadj + eis[u]) : make_int2(0, 0);
                            }
#pragma unroll
                            for (int u = 0; u < kPprBatchUnroll; ++u) {
                                const unsigned pk = (unsigned)__shfl_sync(kFull, (int)qpk, js[u]);
                                DSplit sj;
                                sj.lo = (unsigned)__shfl_sync(kFull, (int)qs.lo, js[u]);
                                sj.hi = pk & 0x1fffffu;
                                sj.e = (int)(pk >> 21);
                                const int qq = __shfl_sync(kFull, qp, js[u]);
                                const unsigned wb = (unsigned)ew[u].y;
                                // m = qu * w in FP64, on the integer pipes (fp64_mul.h)
                                bool send = ok[u] && (int)wb > 0;
                                const bool mok = pk != 0u && c2g_mul_w_ok(wb);
                                double m = c2g_mul(sj, wb);
                                const bool slow = __any_sync(kFull, send && !mok);
                                if (slow) {  // w subnormal: FP64 pipe
                                    const double quj = __shfl_sync(kFull, qu, js[u]);
                                    if (!mok) m = quj * (double)__uint_as_float(wb);
                                    send = send && (mok || m > 0.0);
                                }
                                const size_t tv = (size_t)(unsigned)ew[u].x;
                                if (send) atomicAdd(mw + tv * Qu + qq, m);
                                // Touched lanes: every active query sends along a positive
                                // weight, so slot 0 marks the whole word at once.
                                if (!slow) {
                                    if (send && js[u] == 0) atomicOr(trow + (tv << p.logW), km);
                                } else if (send) {
                                    atomicOr(trow + (tv << p.logW), 1u << qq);
                                }
                            }
                        });
                        if (lane == 0) pushes += (long long)cnt * len;
                        steps += len;
                    }
                    e0 = seg_end;
                    o += 32;
                }
            }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tph, 2);
        if (gtid == 0) trace_mid(p.trace, iters - 1);
        // The frontier just consumed leaves the pull lookup.
        for (unsigned j = gtid; j < F; j += nthreads) p.amask[buf][ldcg(p.q[buf] + j).x] = 0u;
        // Phase B: apply the messages of the touched pairs and activate: after a pull, the
        // listed straddlers (unless the list overflowed); after a push, every touched word.
        const unsigned nl = pull ? ldcg(&ctl->listctr[cur % 3]) : 0u;
        const bool listed = pull && nl <= p.slist_cap;  // grid-uniform
        touched += pbatch_sweep(p, false, ob, listed ? p.slist : nullptr, nl, fst, pbatch_out(p, ob, nslot),
                                &ctl->dctr[nslot], psum, gwarp, nwarps, lane);
        if (lane == 0 && psum) atomicAdd(&ctl->pcount[nslot], psum);
        psum = 0;
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tph, 1);
        ++cur;
    }
    if (bad) atomicOr(flags, C2G_FLAG_BOUNDS);
    // pushes are counted by lane 0 of each warp; touched lanes by every lane
    unsigned long long tl = touched;
    for (int o = 16; o >= 1; o >>= 1) tl += __shfl_xor_sync(kFull, tl, o);
    if (lane == 0) {
        atomicAdd((unsigned long long*)&p.counters[0], (unsigned long long)pushes);
        atomicAdd((unsigned long long*)&p.counters[1], (unsigned long long)steps);
        atomicAdd((unsigned long long*)&ctl->touched, tl);
    }
    if (gtid == 0) {
        ctl->iterations = iters;
        trace_round(p.trace, iters, 0, -1);
    }
}

// [V][Q] float -> caller layout (first nq queries).
__global__ void batch_transpose_f(const float* __restrict__ src, int V, int Q, int nq, float* __restrict__ out,
                                  int query_major) {
    const size_t total = (size_t)V * (size_t)nq;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        if (query_major) {
            const size_t qi = i / (size_t)V, v = i % (size_t)V;
            out[i] = src[v * Q + qi];
        } else {
            const size_t v = i / (size_t)nq, qi = i % (size_t)nq;
            out[i] = src[v * Q + qi];
        }
    }
}

// [V][Q] double -> caller layout as float (first nq queries).
__global__ void batch_transpose_d2f(const double* __restrict__ src, int V, int Q, int nq, float* __restrict__ out,
                                    int query_major) {
    const size_t total = (size_t)V * (size_t)nq;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        if (query_major) {
            const size_t qi = i / (size_t)V, v = i % (size_t)V;
            out[i] = (float)src[v * Q + qi];
        } else {
            const size_t v = i / (size_t)nq, qi = i % (size_t)nq;
            out[i] = (float)src[v * Q + qi];
        }
    }
}

struct PprBatchWork {
    float* pr = nullptr;
    double* res = nullptr;
    double* msg = nullptr;
    double* rq = nullptr;
    double* rq2 = nullptr;
    float2* rqf[2] = {nullptr, nullptr};
    unsigned* amask[2] = {nullptr, nullptr};
    unsigned* tmask = nullptr;
    unsigned* slist = nullptr;
    unsigned slist_cap = 0;
    unsigned* dmask = nullptr;
    int2* q[2] = {nullptr, nullptr};
    unsigned* qmask[2] = {nullptr, nullptr};
    int* mark[2] = {nullptr, nullptr};
    int2* dangle = nullptr;
    TraversalCtl* ctl = nullptr;
    long long* counters = nullptr;
    int* src = nullptr;
    int* seed_off = nullptr;
    int* seed_v = nullptr;
    float* seed_w = nullptr;
    float* stage = nullptr;
    RoundTrace* trace = nullptr;
    size_t seed_cap = 0;
    int Q = 0;
    bool clean = false;  // msg, tmask and amask are zero
};

void ppr_batch_free(c2g_graph* g) {
    PprBatchWork* w = reinterpret_cast<PprBatchWork*>(g->ppr_batch);
    if (!w) return;
    if (g->last_trace == w->trace) g->last_trace = nullptr;
    void* ptrs[] = {w->pr, w->res, w->msg, w->rq, w->rq2, w->rqf[0], w->rqf[1], w->amask[0], w->amask[1], w->tmask,
                    w->slist, w->dmask,
                    w->q[0], w->q[1],
                    w->qmask[0], w->qmask[1],
                    w->mark[0], w->mark[1], w->dangle, w->ctl, w->counters, w->src, w->seed_off,
                    w->seed_v, w->seed_w, w->stage, w->trace};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    delete w;
    g->ppr_batch = nullptr;
}

static int ppr_batch_alloc(c2g_graph* g, int Q, size_t n_seeds) {
    PprBatchWork* w = reinterpret_cast<PprBatchWork*>(g->ppr_batch);
    if (w && w->Q >= Q && w->seed_cap >= n_seeds) return C2G_OK;
    if (w) ppr_batch_free(g);
    w = new PprBatchWork();
    g->ppr_batch = w;
    const size_t V = g->V ? (size_t)g->V : 1;
    const size_t W = (size_t)Q / 32, VQ = V * (size_t)Q;
    const size_t qcap = V * W;
    const size_t mark_cap = (((size_t)g->E * W) >> kBatchTileLog) + 2;
    C2G_CUDA(cudaMalloc(&w->pr, sizeof(float) * VQ));
    C2G_CUDA(cudaMalloc(&w->res, sizeof(double) * VQ));
    C2G_CUDA(cudaMalloc(&w->msg, sizeof(double) * VQ));
    C2G_CUDA(cudaMalloc(&w->rq, sizeof(double) * VQ));
    C2G_CUDA(cudaMalloc(&w->rq2, sizeof(double) * VQ));
    C2G_CUDA(cudaMalloc(&w->rqf[0], sizeof(float2) * VQ));
    C2G_CUDA(cudaMalloc(&w->rqf[1], sizeof(float2) * VQ));
    C2G_CUDA(cudaMalloc(&w->tmask, sizeof(unsigned) * qcap));
    // pull rounds' straddlers: at most one owner per in-edge tile boundary, W words each
    const size_t ntiles_r = (((size_t)g->E + (1u << kPullTileLog) - 1) >> kPullTileLog) + 1;
    w->slist_cap = (unsigned)std::min(qcap, ntiles_r * W);
    C2G_CUDA(cudaMalloc(&w->slist, sizeof(unsigned) * w->slist_cap));
    C2G_CUDA(cudaMalloc(&w->dmask, sizeof(unsigned) * qcap));
    C2G_CUDA(cudaMalloc(&w->amask[0], sizeof(unsigned) * qcap));
    C2G_CUDA(cudaMalloc(&w->amask[1], sizeof(unsigned) * qcap));
    for (int b = 0; b < 2; ++b) {
        C2G_CUDA(cudaMalloc(&w->q[b], sizeof(int2) * qcap));
        C2G_CUDA(cudaMalloc(&w->qmask[b], sizeof(unsigned) * qcap));
        C2G_CUDA(cudaMalloc(&w->mark[b], sizeof(int) * mark_cap));
    }
    C2G_CUDA(cudaMalloc(&w->dangle, sizeof(int2) * qcap));
    C2G_CUDA(cudaMalloc(&w->ctl, sizeof(TraversalCtl)));
    C2G_CUDA(cudaMalloc(&w->counters, sizeof(long long) * 2));
    C2G_CUDA(cudaMalloc(&w->src, sizeof(int) * (size_t)Q));
    C2G_CUDA(cudaMalloc(&w->seed_off, sizeof(int) * ((size_t)Q + 1)));
    w->seed_cap = n_seeds > 0 ? n_seeds : 1;
    C2G_CUDA(cudaMalloc(&w->seed_v, sizeof(int) * w->seed_cap));
    C2G_CUDA(cudaMalloc(&w->seed_w, sizeof(float) * w->seed_cap));
    C2G_CUDA(cudaMalloc(&w->trace, sizeof(RoundTrace) * (kMaxTraceRounds + 1)));
    w->Q = Q;
    w->clean = false;
    return C2G_OK;
}

// Largest positive weight of the reverse CSR (its bits: positive floats order as
// integers).  A non-finite weight makes it non-finite, which disables pull rounds.
__global__ void weight_stats_kernel(const int2* __restrict__ adj_r, long long E, unsigned* wmax_bits) {
    unsigned wm = 0;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < E; e += (long long)gridDim.x * blockDim.x) {
        const int wb = __ldg(adj_r + e).y;
        if (wb > 0) wm = max(wm, (unsigned)wb);
    }
    for (int o = 16; o >= 1; o >>= 1) wm = max(wm, (unsigned)__shfl_xor_sync(kFull, (int)wm, o));
    if ((threadIdx.x & 31) == 0 && wm) atomicMax(wmax_bits, wm);
}

// Reverse CSR and weight statistics for pull rounds (once per graph and weights).
int ppr_pull_prepare(c2g_graph* g) {
    int rc = build_reverse_graph(g);
    if (rc || g->wstat_valid) return rc;
    unsigned* d = nullptr;
    C2G_CUDA(cudaMalloc(&d, sizeof(unsigned)));
    cudaError_t e = cudaMemsetAsync(d, 0, sizeof(unsigned), g->stream);
    if (e == cudaSuccess && g->E > 0) {
        weight_stats_kernel<<<g->num_sms * 8, 256, 0, g->stream>>>(g->adj_r, (long long)g->E, d);
        e = cudaGetLastError();
    }
    unsigned h = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(&h, d, sizeof(unsigned), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(d);
    C2G_CUDA(e);
    g->wstat_wmax_bits = h;
    g->wstat_valid = true;
    return C2G_OK;
}

// Push count above which a round pulls (c2g_ppr_batch_set_pull): pull rounds need the
// reverse CSR (a view uses its base's, never builds it) and finite weights; with rmax
// below 1e-30 pushed residuals may leave the FP32 range of the pull's float pairs, so such
// launches push only.
static int ppr_pull_threshold(c2g_graph* g, const c2g_ppr_params& prm, unsigned long long* pull_min) {
    *pull_min = ~0ull;
    const float ratio = g->ppr_cfg.batch_pull_ratio;
    if (ratio >= 0.f && g->E > 0 && prm.rmax >= 1e-30f && (g->wstat_valid || !g->borrowed)) {
        int rc;
        if (!g->borrowed && (rc = ppr_pull_prepare(g))) return rc;
        float wmax;
        std::memcpy(&wmax, &g->wstat_wmax_bits, sizeof(float));
        if (std::isfinite(wmax)) *pull_min = (unsigned long long)((double)ratio * (double)g->E);
    }
    return C2G_OK;
}

// msg, tmask, dmask and both activity masks are zero between launches.
static int ppr_batch_clean(c2g_graph* g, PprBatchWork* w) {
    if (w->clean) return C2G_OK;
    const size_t VQ = (size_t)g->V * (size_t)w->Q;
    C2G_CUDA(cudaMemsetAsync(w->msg, 0, sizeof(double) * VQ, g->stream));
    for (unsigned* m : {w->tmask, w->dmask, w->amask[0], w->amask[1]})
        C2G_CUDA(cudaMemsetAsync(m, 0, sizeof(unsigned) * (size_t)g->V * (size_t)(w->Q / 32), g->stream));
    w->clean = true;
    return C2G_OK;
}

static void ppr_batch_params(c2g_graph* g, PprBatchWork* w, int Q, int logW, const c2g_ppr_params& prm,
                             unsigned long long pull_min, PprBatchParams& p) {
    const int nq = Q;
    const std::vector<int32_t>* seed_off = nullptr;
    p.row = g->row;
    p.adj = g->adj_f;
    p.E = (unsigned)g->E;
    p.V = g->V;
    p.logW = logW;
    p.Q = Q;
    p.nq = nq;
    p.pr = w->pr;
    p.res = w->res;
    p.msg = w->msg;
    p.rq[0] = w->rq;
    p.rq[1] = w->rq2;
    p.amask[0] = w->amask[0];
    p.amask[1] = w->amask[1];
    p.rqf[0] = w->rqf[0];
    p.rqf[1] = w->rqf[1];
    p.tmask = w->tmask;
    p.slist = w->slist;
    p.slist_cap = w->slist_cap;
    p.dmask = w->dmask;
    p.epoch_rounds = 0;
    p.cur0 = 1;
    for (int b = 0; b < 2; ++b) {
        p.q[b] = w->q[b];
        p.qmask[b] = w->qmask[b];
        p.mark[b] = w->mark[b];
    }
    p.dangle = w->dangle;
    p.ctl = w->ctl;
    p.sources = w->src;
    p.seed_off = seed_off ? w->seed_off : nullptr;
    p.seed_v = w->seed_v;
    p.seed_w = w->seed_w;
    p.alpha = prm.alpha;
    p.rmax = prm.rmax;
    p.r0 = prm.r0;
    p.pr0 = prm.pr0;
    p.seeded = prm.seeded;
    p.max_iter = prm.max_iter;
    p.qcap = (unsigned)((size_t)g->V * (size_t)(p.Q / 32));
    p.mark_cap = (unsigned)((((size_t)g->E * (size_t)(p.Q / 32)) >> kBatchTileLog) + 2);
    p.barrier_ns = g->barrier_ns ? g->barrier_ns : 4000000000ull;
    p.counters = w->counters;
    p.row_r = g->row_r;
    p.adj_r = g->adj_r;
    p.mark_r = g->mark_r;
    p.ntiles_r = (unsigned)(((size_t)g->E + (1u << kPullTileLog) - 1) >> kPullTileLog);
    p.pull_min = pull_min;
    p.trace = w->trace;
    g->last_trace = w->trace;
}

int ppr_batch_launch(c2g_graph* g, int32_t nq, const int32_t* sources, const c2g_ppr_params& prm,
                     const std::vector<int32_t>* seed_off, const std::vector<int32_t>* seed_v,
                     const std::vector<float>* seed_w, float* pr_out, float* res_out, int on_device, int query_major,
                     float* ms, long long* counters, TraversalCtl* ctl_out) {
    if (!g->adj_f) return fail(C2G_ERR_UNSUPPORTED, "graph has no float weights (flist / ppr wlist)");
    int Q = 32, logW = 0;
    while (Q < nq) {
        Q <<= 1;
        ++logW;
    }
    if ((size_t)g->V * (size_t)(Q / 32) >= (size_t(1) << 31) || (size_t)g->E * (size_t)(Q / 32) >= (size_t(1) << 32))
        return fail(C2G_ERR_RANGE, "batch of %d queries too large for this graph", nq);
    int rc;
    const size_t ns = seed_v ? seed_v->size() : 0;
    unsigned long long pull_min = ~0ull;
    if ((rc = ppr_pull_threshold(g, prm, &pull_min))) return rc;
    if ((rc = ppr_batch_alloc(g, Q, ns))) return rc;
    PprBatchWork* w = reinterpret_cast<PprBatchWork*>(g->ppr_batch);
    int coop = 0, per_sm = 0;
    C2G_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, g->device));
    if (!coop) return fail(C2G_ERR_UNSUPPORTED, "device lacks cooperative launch");
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ppr_batch_persistent, kPprBatchThreads, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "batch kernel cannot be resident");
    const size_t VQ = (size_t)g->V * (size_t)w->Q;
    if ((rc = ppr_batch_clean(g, w))) return rc;
    C2G_CUDA(cudaMemcpyAsync(w->src, sources, sizeof(int) * (size_t)nq, cudaMemcpyHostToDevice, g->stream));
    if (seed_off) {
        C2G_CUDA(cudaMemcpyAsync(w->seed_off, seed_off->data(), sizeof(int) * seed_off->size(), cudaMemcpyHostToDevice,
                                 g->stream));
        if (ns) {
            C2G_CUDA(cudaMemcpyAsync(w->seed_v, seed_v->data(), sizeof(int) * ns, cudaMemcpyHostToDevice, g->stream));
            C2G_CUDA(cudaMemcpyAsync(w->seed_w, seed_w->data(), sizeof(float) * ns, cudaMemcpyHostToDevice, g->stream));
        }
    }
    PprBatchParams p;
    ppr_batch_params(g, w, Q, logW, prm, pull_min, p);
    p.nq = nq;
    p.seed_off = seed_off ? w->seed_off : nullptr;
    C2G_CUDA(cudaMemsetAsync(w->ctl, 0, sizeof(TraversalCtl), g->stream));
    C2G_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(long long) * 2, g->stream));
    void* args[] = {&p};
    C2G_CUDA(cudaEventRecord(g->ev0, g->stream));
    const int blocks = grid_blocks(g, per_sm);
    C2G_CUDA(cudaLaunchCooperativeKernel((const void*)ppr_batch_persistent, dim3(blocks), dim3(kPprBatchThreads), args,
                                         0, g->stream));
    C2G_CUDA(cudaEventRecord(g->ev1, g->stream));
    cudaError_t e = cudaSuccess;
    float* outs[2] = {pr_out, res_out};
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        if (!outs[k]) continue;
        float* dst = outs[k];
        float* direct = on_device ? nullptr : static_cast<float*>(mapped_host(outs[k]));
        if (direct) {
            dst = direct;
        } else if (!on_device) {
            if (!w->stage) e = cudaMalloc(&w->stage, sizeof(float) * VQ);
            dst = w->stage;
        }
        if (e != cudaSuccess) break;
        if (k == 0)
            if (query_major)
                launch_transpose_qmajor<float, float>(w->pr, g->V, p.Q, nq, dst, g->stream);
            else
                batch_transpose_f<<<g->num_sms * 8, 256, 0, g->stream>>>(w->pr, g->V, p.Q, nq, dst, query_major);
        else
            if (query_major)
                launch_transpose_qmajor<double, float>(w->res, g->V, p.Q, nq, dst, g->stream);
            else
                batch_transpose_d2f<<<g->num_sms * 8, 256, 0, g->stream>>>(w->res, g->V, p.Q, nq, dst, query_major);
        e = cudaGetLastError();
        if (e == cudaSuccess && !on_device && !direct)
            e = cudaMemcpyAsync(outs[k], dst, sizeof(float) * (size_t)g->V * (size_t)nq, cudaMemcpyDeviceToHost,
                                g->stream);
    }
    if (e == cudaSuccess) e = cudaMemcpyAsync(ctl_out, w->ctl, sizeof(TraversalCtl), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(counters, w->counters, sizeof(long long) * 2, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    C2G_CUDA(e);
    if (ctl_out->flags & (C2G_FLAG_BARRIER_TIMEOUT | C2G_FLAG_QUEUE_OVERFLOW | C2G_FLAG_BOUNDS)) w->clean = false;
    C2G_CUDA(cudaEventElapsedTime(ms, g->ev0, g->ev1));
    return C2G_OK;
}

// Resident batch (c2g_session): the workspace of Q query slots with every array at rest
// (pr, res, msg and the masks zero), its arrays, and one epoch of at most `rounds` rounds
// starting at round cur0 from the state the previous epoch (and the joins since) left.
int ppr_batch_reserve(c2g_graph* g, int Q, PprBatchArrays* a) {
    if (!g->adj_f) return fail(C2G_ERR_UNSUPPORTED, "graph has no float weights (flist / ppr wlist)");
    if ((size_t)g->V * (size_t)(Q / 32) >= (size_t(1) << 31) || (size_t)g->E * (size_t)(Q / 32) >= (size_t(1) << 32))
        return fail(C2G_ERR_RANGE, "%d slots too many for this graph", Q);
    int rc;
    if ((rc = ppr_batch_alloc(g, Q, 0))) return rc;
    PprBatchWork* w = reinterpret_cast<PprBatchWork*>(g->ppr_batch);
    w->clean = false;
    if ((rc = ppr_batch_clean(g, w))) return rc;
    const size_t VQ = (size_t)g->V * (size_t)w->Q;
    C2G_CUDA(cudaMemsetAsync(w->pr, 0, sizeof(float) * VQ, g->stream));
    C2G_CUDA(cudaMemsetAsync(w->res, 0, sizeof(double) * VQ, g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    a->pr = w->pr;
    a->res = w->res;
    a->rq[0] = w->rq;
    a->rq[1] = w->rq2;
    a->rqf[0] = w->rqf[0];
    a->rqf[1] = w->rqf[1];
    a->amask[0] = w->amask[0];
    a->amask[1] = w->amask[1];
    a->dmask = w->dmask;
    return C2G_OK;
}

int ppr_batch_epoch(c2g_graph* g, int Q, const c2g_ppr_params& prm, int cur0, int rounds, float* ms,
                    long long* counters, TraversalCtl* ctl_out) {
    PprBatchWork* w = reinterpret_cast<PprBatchWork*>(g->ppr_batch);
    if (!w || w->Q < Q) return fail(C2G_ERR_ARG, "resident PPR batch has no workspace");
    int logW = 0;
    while ((32 << logW) < Q) ++logW;
    int rc;
    unsigned long long pull_min = ~0ull;
    if ((rc = ppr_pull_threshold(g, prm, &pull_min))) return rc;
    int per_sm = 0;
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ppr_batch_persistent, kPprBatchThreads, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "batch kernel cannot be resident");
    PprBatchParams p;
    ppr_batch_params(g, w, Q, logW, prm, pull_min, p);
    p.epoch_rounds = rounds < 1 ? 1 : rounds;
    p.cur0 = cur0;
    p.max_iter = 1 << 30;  // the per-query caps are the session's
    C2G_CUDA(cudaMemsetAsync(w->ctl, 0, sizeof(TraversalCtl), g->stream));
    C2G_CUDA(cudaMemsetAsync(w->counters, 0, sizeof(long long) * 2, g->stream));
    void* args[] = {&p};
    C2G_CUDA(cudaEventRecord(g->ev0, g->stream));
    C2G_CUDA(cudaLaunchCooperativeKernel((const void*)ppr_batch_persistent, dim3(grid_blocks(g, per_sm)),
                                         dim3(kPprBatchThreads), args, 0, g->stream));
    C2G_CUDA(cudaEventRecord(g->ev1, g->stream));
    C2G_CUDA(cudaMemcpyAsync(ctl_out, w->ctl, sizeof(TraversalCtl), cudaMemcpyDeviceToHost, g->stream));
    C2G_CUDA(cudaMemcpyAsync(counters, w->counters, sizeof(long long) * 2, cudaMemcpyDeviceToHost, g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    C2G_CUDA(cudaEventElapsedTime(ms, g->ev0, g->ev1));
    return C2G_OK;
}

}  // namespace c2g
