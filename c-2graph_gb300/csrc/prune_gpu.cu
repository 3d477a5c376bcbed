// purn-ppr (src/purn-ppr.cpp:63-344) and purn-sssp (src/purn-sssp.cpp:61-352) on the GPU,
// writing the same bytes as the host passes (prune.cpp) and the reference.
//
// Both pruners visit vertices in a fixed order: purn-ppr every vertex once in id order with
// the in-degree bound 5; purn-sssp in rounds k = 1..29, each over the vertices in id order,
// visiting a vertex in the first round whose bound k covers its live in-degree.  Call the
// steps of that order positions (k, i).  A visit of i with out-edges moves each out-edge
// i -> v that every live in-neighbour ("root") of i but at most one already has into the
// roots' rows, with folded weights, and records it.  A position reads i's in-row (its
// live in-degree and roots), i's out-row and its roots' out-rows; a visit that moves edges
// writes i's out-row, its roots' out-rows and the in-rows of the moved targets.  So the
// order matters only between positions that share rows.
//
// The device pruner runs the positions in rounds of a speculative schedule (deterministic
// reservations).  Every round, every pending position of a window plans its step on the
// current state (the rows it reads and would write, and which out-edges move) and reserves
// those rows under its index.  It commits when no earlier position of the window writes a
// row it reads or touches a row it writes.  A position with an earlier writer of a row it
// reads may see its plan change before it commits, and so may the rows it will touch, so
// nothing past the first such position commits in the round.  The first pending position
// always commits, so every round makes progress.  A window holds at
// most V positions, so no vertex appears in it twice.  The schedule is the one
// orc_prune_speculative runs on the CPU (the same rounds, the same bytes).  A position that
// only decides (its vertex is not pruned at its turn) is handled by one lane; a position
// that prunes by a warp.
//
// Committed visits touch disjoint rows and run in parallel, one warp each, with the
// reference's steps: roots in in-row order; the out-row split into kept pairs (compacted
// in place) and moved pairs (the record); each moved target's in-row gains the roots that
// lack the target (a revived entry, or an inserted one) and loses i; the moved pairs merge
// into each root's sorted row (a pair whose target the row has folds into it, a new target
// is inserted with the folded weight).  Updates of existing entries are made in place.  A
// row that gains entries moves to a new block of its pool (bump allocation): the visit
// writes the new entries there and queues the old row's segments between them as copy
// tasks of at most kPgTask entries, which the whole grid runs after the commit phase, so
// the copying of long rows (hubs are the roots of many pruned vertices) is spread over
// every SM instead of one warp.
#include <algorithm>
#include <cstring>
#include <string>
#include <type_traits>
#include <vector>

#include "../../include/c2graph.h"
#include "device_common.cuh"
#include "host_io.h"
#include "internal.h"

namespace c2g {

template <typename W>
int prune_initial_rows(const std::string& dir, int32_t& V, std::vector<int32_t>& orow, std::vector<int32_t>& ot,
                       std::vector<W>& ow, std::vector<int32_t>& irow, std::vector<int32_t>& is);

constexpr int kPgThreads = 256;
constexpr int kPgWarps = kPgThreads / 32;
constexpr int kPgSlotR = 32;   // rows a position reads: its in-row, its out-row, its roots' out-rows
constexpr int kPgG = 6;        // roots searched in lockstep
constexpr int kPgU = 2;        // merge items per lane searched in lockstep
constexpr int kPgTask = 1024;  // entries per copy task
constexpr unsigned kPgMoved = 0x80000000u;  // plan code of an out-edge that moves (| the roots lacking it)

// Fold rules (src/purn-ppr.cpp:244,255,259; src/purn-sssp.cpp:244,255,263).  Weights are
// 32-bit patterns: float for purn-ppr, int32 for purn-sssp.  d3 is the moved pair's
// weight, dis the weight of root -> i.
struct PgPpr {
    static constexpr int kMaxRoots = 5;
    // (float * keep) * float evaluated in double, rounded to float
    static __device__ __forceinline__ unsigned fold_new(unsigned d3, unsigned dis, double keep) {
        return __float_as_uint(__double2float_rn(
            __dmul_rn(__dmul_rn((double)__uint_as_float(d3), keep), (double)__uint_as_float(dis))));
    }
    static __device__ __forceinline__ unsigned fold_hit(unsigned old, unsigned d3, unsigned dis, double keep) {
        const double f = __dmul_rn(__dmul_rn((double)__uint_as_float(d3), keep), (double)__uint_as_float(dis));
        return __float_as_uint(__double2float_rn(__dadd_rn((double)__uint_as_float(old), f)));
    }
};
struct PgSssp {
    static constexpr int kMaxRoots = 29;
    // int32 sums wrap as the reference's do; a fold into an existing pair keeps the minimum
    static __device__ __forceinline__ unsigned fold_new(unsigned d3, unsigned dis, double) { return d3 + dis; }
    static __device__ __forceinline__ unsigned fold_hit(unsigned old, unsigned d3, unsigned dis, double) {
        return (unsigned)min((int)old, (int)(d3 + dis));
    }
};

struct PgCtl {
    unsigned bar_count, bar_gen;  // GridBarrier
    int flags;
    unsigned pos;      // the window's first position
    unsigned dmin;     // this round: the first position with an earlier writer of a row it reads
    unsigned nextpos;  // this round: the first position left pending
    int round;
    int finished;
    unsigned long long out_top, in_top, rec_top, wscr_top, mscr_top;  // pool bump pointers
    unsigned long long task_top[2];                                   // copy tasks, by round parity
    unsigned long long phase_ns[4];  // block 0's time in plan, check, commit, copy (waits included)
};

struct PgTask {
    long long src, dst;
    int len, kind;  // kind 0: out-row pairs (ot, ow); 1: in-row entries (is, ia)
};

struct PgParams {
    int V;
    int kfirst, klast;  // positions (k, i): k = kfirst..klast, i = 0..V-1; index (k - kfirst) * V + i
    unsigned npos;
    double keep;
    int span;  // window: positions pos .. pos + span - 1
    long long* out_off;
    int* out_n;
    int* ot;
    unsigned* ow;
    unsigned long long out_cap;
    long long* in_off;
    int* in_n;
    int* is;
    unsigned char* ia;  // alive flags of the in-row entries
    unsigned long long in_pool_cap;
    int* indeg;
    int* pk;  // per vertex: the last round whose position is done (klast once visited)
    int* vk;  // per vertex: the round of its pruning visit, 0 if none
    long long* rec_off;
    int* rec_n;
    int* rt;
    unsigned* rw;
    unsigned* rmiss;  // per moved pair: the roots (bits, root order) without its target
    unsigned long long rec_cap;
    unsigned long long* resA;  // [2V] (round << 32) | ~position, the earliest position touching the row
    unsigned long long* resW;  // [2V] the same for writers
    int* slot_r;               // [span][kPgSlotR] rows read (out-row x is x, in-row x is V + x)
    int* slot_rn;              // rows read, -1: the position was done before the round
    long long* slot_woff;      // plan block in wscr: rows written, then one code per out-edge
    int* slot_wn;
    unsigned char* slot_pass;
    int* wscr;
    unsigned long long wscr_cap;
    int* mscr;  // merge scratch of the committing visits
    unsigned long long mscr_cap;
    PgTask* task;
    unsigned long long task_cap;
    PgCtl* ctl;
    unsigned long long barrier_ns;
    int max_rounds;
};

constexpr int kPgErrPool = C2G_FLAG_QUEUE_OVERFLOW;  // a pool ran out
constexpr int kPgErrRows = C2G_FLAG_BOUNDS;          // rows disagree (in-row without its out-edge)

// State that other SMs change between rounds is read from L2 (ld.global.cg), never from a
// possibly stale L1 line.
__device__ __forceinline__ long long ldl(const long long* q) { return __ldcg(q); }
__device__ __forceinline__ unsigned char ldb(const unsigned char* q) { return __ldcg(q); }

__device__ __forceinline__ unsigned long long pg_key(int round, unsigned pos) {
    return ((unsigned long long)(unsigned)round << 32) | (unsigned long long)(~pos);
}

// A vertex's live roots in in-row order with their out-rows, per warp in shared memory.
struct PgRoots {
    int j;
    int r[32];
    int n[32];
    long long off[32];
    unsigned dis[32];  // weight of root -> i
    int nnew[32];      // merge: new pairs per root
};

// The live roots of i.  Returns their count (a count above MAXR may stop early); S.j keeps
// the first min(count, MAXR).
template <int MAXR>
__device__ __forceinline__ int pg_roots(const PgParams& p, int i, PgRoots& S, int lane) {
    const long long off = ldl(p.in_off + i);
    const int n = ldcg(p.in_n + i);
    int nr = 0;
    for (int b = 0; b < n && nr <= MAXR; b += 32) {
        const int k = b + lane;
        const bool a = k < n && ldb(p.ia + off + k) != 0;
        const int s = k < n ? ldcg(p.is + off + k) : 0;
        const unsigned m = __ballot_sync(kFull, a);
        const int at = nr + __popc(m & ((1u << lane) - 1u));
        if (a && at < 32) S.r[at] = s;
        nr += __popc(m);
    }
    const int j = min(nr, MAXR);
    if (lane == 0) S.j = j;
    __syncwarp();
    if (lane < j) {
        S.off[lane] = ldl(p.out_off + S.r[lane]);
        S.n[lane] = ldcg(p.out_n + S.r[lane]);
    }
    __syncwarp();
    return nr;
}

// Does the edge i -> v move (every root but at most one has v)?  miss: roots without v.
// Membership in a root's sorted row is the reference's monotone cursor test
// (src/purn-ppr.cpp:170-186, src/purn-sssp.cpp:195-205) as a lower bound; kPgG roots'
// searches run in lockstep.
__device__ __forceinline__ bool pg_moves(const PgParams& p, const PgRoots& S, int j, int v, unsigned& miss) {
    miss = 0u;
    for (int k = 0; k < j; ++k)
        if (S.r[k] == v) return false;  // a root keeps its edge
    unsigned has = 0u;
    for (int g = 0; g < j; g += kPgG) {
        int lo[kPgG], hi[kPgG];
        long long off[kPgG];
#pragma unroll
        for (int u = 0; u < kPgG; ++u) {
            const int k = g + u;
            lo[u] = 0;
            hi[u] = k < j ? S.n[k] : 0;
            off[u] = k < j ? S.off[k] : 0;
        }
        for (;;) {
            int t[kPgG];
            bool any = false;
#pragma unroll
            for (int u = 0; u < kPgG; ++u) {
                t[u] = 0;
                if (lo[u] < hi[u]) {
                    t[u] = ldcg(p.ot + off[u] + ((lo[u] + hi[u]) >> 1));
                    any = true;
                }
            }
            if (!any) break;
#pragma unroll
            for (int u = 0; u < kPgG; ++u)
                if (lo[u] < hi[u]) {
                    const int mid = (lo[u] + hi[u]) >> 1;
                    if (t[u] < v)
                        lo[u] = mid + 1;
                    else
                        hi[u] = mid;
                }
        }
#pragma unroll
        for (int u = 0; u < kPgG; ++u) {
            const int k = g + u;
            if (k < j && lo[u] < S.n[k] && ldcg(p.ot + off[u] + lo[u]) == v) has |= 1u << k;
        }
    }
    miss = ((1u << j) - 1u) & ~has;
    return __popc(has) + 2 > j;
}

// Does the step at round k visit i and prune it (live in-degree in [1, k], out-edges)?
__device__ __forceinline__ bool pg_prunes(const PgParams& p, int i, int k) {
    const int d = ldcg(p.indeg + i);
    return d > 0 && d <= k && ldcg(p.out_n + i) > 0;
}

// Queue the copy of `len` entries from src to dst (pool indices) as tasks.
__device__ __forceinline__ void pg_emit(const PgParams& p, int par, int kind, long long src, long long dst,
                                        long long len) {
    for (long long x = 0; x < len; x += kPgTask) {
        const unsigned long long t = atomicAdd(&p.ctl->task_top[par], 1ull);
        if (t >= p.task_cap) {
            atomicOr(&p.ctl->flags, kPgErrPool);
            return;
        }
        PgTask* tk = p.task + t;
        tk->src = src + x;
        tk->dst = dst + x;
        tk->len = (int)min((long long)kPgTask, len - x);
        tk->kind = kind;
    }
}

// Plan of position pos = (k, i) (slot c): the rows it reads, the rows it would write, and
// per out-edge whether it moves; reserve the rows.  The plan block in wscr holds the
// written rows (at most on + 30) in [0, on + 32) and the out-edge codes in
// [on + 32, 2 on + 32).
template <typename Rule>
__device__ __forceinline__ void pg_plan(const PgParams& p, unsigned pos, int i, int k, int c, int round, int lane,
                                        PgRoots& S) {
    const int V = p.V;
    int* Rw = p.slot_r + (size_t)c * kPgSlotR;
    int rn = 2;
    if (lane == 0) {
        Rw[0] = V + i;
        Rw[1] = i;
    }
    long long woff = 0;
    int wn = 0;
    if (pg_prunes(p, i, k)) {
        pg_roots<Rule::kMaxRoots>(p, i, S, lane);
        const int j = S.j;
        if (lane < j) Rw[2 + lane] = S.r[lane];
        rn = 2 + j;
        const long long off = ldl(p.out_off + i);
        const int on = ldcg(p.out_n + i);
        const unsigned long long need = 2ull * (unsigned long long)on + 32ull;
        unsigned long long wb = 0;
        if (lane == 0) wb = atomicAdd(&p.ctl->wscr_top, need);
        wb = __shfl_sync(kFull, wb, 0);
        if (wb + need > p.wscr_cap) {
            if (lane == 0) atomicOr(&p.ctl->flags, kPgErrPool);
        } else {
            woff = (long long)wb;
            int* code = p.wscr + woff + on + 32;
            for (int b = 0; b < on; b += 32) {
                const int e = b + lane;
                unsigned miss = 0u;
                const int v = e < on ? ldcg(p.ot + off + e) : 0;
                const bool mv = e < on && pg_moves(p, S, j, v, miss);
                if (e < on) code[e] = mv ? (int)(kPgMoved | miss) : 0;
                const unsigned m = __ballot_sync(kFull, mv);
                if (mv) p.wscr[woff + wn + __popc(m & ((1u << lane) - 1u))] = V + v;
                wn += __popc(m);
            }
            if (wn > 0) {  // it moves edges: its out-row and its roots' out-rows change
                if (lane == 0) p.wscr[woff + wn] = i;
                if (lane < j) p.wscr[woff + wn + 1 + lane] = S.r[lane];
                wn += 1 + j;
            }
        }
    }
    if (lane == 0) {
        p.slot_rn[c] = rn;
        p.slot_woff[c] = woff;
        p.slot_wn[c] = wn;
    }
    __syncwarp();
    const unsigned long long key = pg_key(round, pos);
    if (lane < rn) atomicMax(p.resA + Rw[lane], key);
    for (int x = lane; x < wn; x += 32) {
        const int r = p.wscr[woff + x];
        atomicMax(p.resA + r, key);
        atomicMax(p.resW + r, key);
    }
}

// v's in-row after the `cnt` moved pairs i -> v of a visit (one lane): every root in `miss`
// gets a live entry (revived, or inserted in source order) and counts in v's in-degree, and
// i's entry dies once per pair (src/purn-ppr.cpp:196-236, src/purn-sssp.cpp:207-242).
template <typename Rule>
__device__ __forceinline__ void pg_in_update(const PgParams& p, const PgRoots& S, int j, int i, int v, unsigned miss,
                                             int cnt, int par) {
    const long long off = ldl(p.in_off + v);
    const int n = ldcg(p.in_n + v);
    int qi = n, inc = 0, nins = 0;
    int at_l[Rule::kMaxRoots], who_l[Rule::kMaxRoots];
    for (int g = 0; g < j; g += kPgG) {
        // lockstep lower bounds of the group's missing roots (and of i, with the first group)
        int lo[kPgG + 1], hi[kPgG + 1], key[kPgG + 1];
#pragma unroll
        for (int u = 0; u < kPgG; ++u) {
            const int k = g + u;
            const bool use = k < j && ((miss >> k) & 1u);
            key[u] = use ? S.r[k] : 0;
            lo[u] = 0;
            hi[u] = use ? n : 0;
        }
        key[kPgG] = i;
        lo[kPgG] = 0;
        hi[kPgG] = g == 0 ? n : 0;
        for (;;) {
            int t[kPgG + 1];
            bool any = false;
#pragma unroll
            for (int u = 0; u <= kPgG; ++u) {
                t[u] = 0;
                if (lo[u] < hi[u]) {
                    t[u] = ldcg(p.is + off + ((lo[u] + hi[u]) >> 1));
                    any = true;
                }
            }
            if (!any) break;
#pragma unroll
            for (int u = 0; u <= kPgG; ++u)
                if (lo[u] < hi[u]) {
                    const int mid = (lo[u] + hi[u]) >> 1;
                    if (t[u] < key[u])
                        lo[u] = mid + 1;
                    else
                        hi[u] = mid;
                }
        }
        if (g == 0) qi = lo[kPgG];
#pragma unroll
        for (int u = 0; u < kPgG; ++u) {
            const int k = g + u;
            if (!(k < j && ((miss >> k) & 1u))) continue;
            const int q = lo[u];
            if (q < n && ldcg(p.is + off + q) == key[u]) {
                if (!ldb(p.ia + off + q)) {
                    p.ia[off + q] = 1;
                    ++inc;
                }
            } else if (nins < Rule::kMaxRoots) {
                at_l[nins] = q;  // roots ascend, so the insertion points do too
                who_l[nins] = key[u];
                ++nins;
                ++inc;
            }
        }
    }
    if (qi >= n || ldcg(p.is + off + qi) != i) {
        atomicOr(&p.ctl->flags, kPgErrRows);
        return;
    }
    p.ia[off + qi] = 0;
    p.indeg[v] = ldcg(p.indeg + v) + inc - cnt;
    if (nins > 0) {
        const unsigned long long nb = atomicAdd(&p.ctl->in_top, (unsigned long long)(n + nins));
        if (nb + (unsigned long long)(n + nins) > p.in_pool_cap) {
            atomicOr(&p.ctl->flags, kPgErrPool);
            return;
        }
        const long long nbo = (long long)nb;
        int prev = 0;
        for (int s = 0; s < nins; ++s) {
            const int at = at_l[s];
            pg_emit(p, par, 1, off + prev, nbo + prev + s, at - prev);
            p.is[nbo + at + s] = who_l[s];
            p.ia[nbo + at + s] = 1;
            prev = at;
        }
        pg_emit(p, par, 1, off + prev, nbo + prev + nins, n - prev);
        p.in_off[v] = nbo;
        p.in_n[v] = n + nins;
    }
}

// A committed pruning visit of vertex i at round k (slot c; the plan's rows are unchanged
// since the plan).
template <typename Rule>
__device__ __forceinline__ void pg_visit(const PgParams& p, int i, int k, int c, int par, int lane, PgRoots& S) {
    const int nr = pg_roots<Rule::kMaxRoots>(p, i, S, lane);
    const int j = S.j;
    if (nr != ldcg(p.indeg + i) || nr > k) {  // the reference stops on this (something error2)
        if (lane == 0) atomicOr(&p.ctl->flags, kPgErrRows);
        return;
    }
    if (lane < j) S.nnew[lane] = 0;
    const long long ooff = ldl(p.out_off + i);
    const int on = ldcg(p.out_n + i);
    const long long woff = ldl(p.slot_woff + c);
    const int wn = ldcg(p.slot_wn + c);
    const int nrm = wn > 0 ? wn - 1 - j : 0;
    const int* code = p.wscr + woff + on + 32;
    unsigned long long rb = 0, mb = 0;
    const unsigned long long mneed = (unsigned long long)(1 + j) * (unsigned long long)nrm;
    if (nrm > 0) {
        if (lane == 0) {
            rb = atomicAdd(&p.ctl->rec_top, (unsigned long long)nrm);
            mb = atomicAdd(&p.ctl->mscr_top, mneed);
        }
        rb = __shfl_sync(kFull, rb, 0);
        mb = __shfl_sync(kFull, mb, 0);
        if (rb + (unsigned long long)nrm > p.rec_cap || mb + mneed > p.mscr_cap) {
            if (lane == 0) atomicOr(&p.ctl->flags, kPgErrPool);
            return;
        }
    }
    __syncwarp();
    // split the out-row: moved pairs to the record (in order), kept ones compacted in place
    int nm = 0, kn = 0;
    for (int b = 0; b < on; b += 32) {
        const int e = b + lane;
        const bool valid = e < on;
        const int v = valid ? ldcg(p.ot + ooff + e) : 0;
        const unsigned w = valid ? ldcg(p.ow + ooff + e) : 0u;
        const unsigned cd = valid ? (unsigned)ldcg(code + e) : 0u;
        const bool mv = (cd & kPgMoved) != 0u;
        const bool kp = valid && !mv;
        const unsigned mm = __ballot_sync(kFull, mv), mk = __ballot_sync(kFull, kp);
        const unsigned lt = (1u << lane) - 1u;
        if (mv) {
            const int x = nm + __popc(mm & lt);
            if (x < nrm) {
                p.rt[rb + x] = v;
                p.rw[rb + x] = w;
                p.rmiss[rb + x] = cd & ~kPgMoved;
            }
        }
        __syncwarp();  // every lane has read its pair before the compaction writes
        if (kp) {
            const long long at = ooff + kn + __popc(mk & lt);
            p.ot[at] = v;
            p.ow[at] = w;
        }
        nm += __popc(mm);
        kn += __popc(mk);
        __syncwarp();
    }
    if (nm != nrm) {
        if (lane == 0) atomicOr(&p.ctl->flags, kPgErrRows);
        return;
    }
    // in-rows of the moved targets: one lane per run of equal targets
    for (int b0 = 0; b0 < nrm; b0 += 32) {
        const int b = b0 + lane;
        if (b >= nrm) continue;
        const int v = ldcg(p.rt + rb + b);
        if (b > 0 && ldcg(p.rt + rb + b - 1) == v) continue;
        int cnt = 1;
        while (b + cnt < nrm && ldcg(p.rt + rb + b + cnt) == v) ++cnt;
        pg_in_update<Rule>(p, S, j, i, v, ldcg(p.rmiss + rb + b), cnt, par);
    }
    __syncwarp();
    // The moved pairs merge into every root's sorted row.  Pass 1 takes every (root, pair)
    // item at once: a pair whose target the row has (the k-th pair of a run of equal targets
    // goes with the row's k-th pair of that target, as the reference's two-cursor merge
    // pairs them) folds into that pair in place; a new one gets its insertion point.  The
    // merge scratch holds each pair's rank in its run, then the items' insertion points (-1:
    // folded in place).  Pass 2 moves each root's row that gains pairs to a new block.
    int* kbs = p.mscr + mb;
    int* insp = kbs + nrm;
    int run = 0;
    for (int b0 = 0; b0 < nrm; b0 += 32) {
        const int b = b0 + lane;
        const bool valid = b < nrm;
        const int tb = valid ? ldcg(p.rt + rb + b) : 0;
        const bool st = valid && (b == 0 || ldcg(p.rt + rb + b - 1) != tb);
        const unsigned sm = __ballot_sync(kFull, st) & ((2u << lane) - 1u);
        const int rs = sm ? b0 + 31 - __clz(sm) : run;  // where this pair's run starts
        run = __shfl_sync(kFull, rs, 31);
        if (valid) kbs[b] = b - rs;
    }
    __syncwarp();
    // Pass 1 with the weights of root -> i (each root's first pair with target i, looked up
    // by lane q0 for root q0): kPgU items per lane and the lookups searched in lockstep.
    const int items = j * nrm;
    for (int i0 = 0; i0 == 0 || i0 < items; i0 += 32 * kPgU) {
        int lo[kPgU + 1], hi[kPgU + 1], key[kPgU + 1], bb[kPgU], qq[kPgU];
        long long off[kPgU + 1];
#pragma unroll
        for (int u = 0; u < kPgU; ++u) {
            const int it = i0 + u * 32 + lane;
            const bool valid = it < items;
            qq[u] = valid ? it / nrm : 0;
            bb[u] = valid ? it - qq[u] * nrm : 0;
            off[u] = S.off[qq[u]];
            lo[u] = 0;
            hi[u] = valid ? S.n[qq[u]] : 0;
            key[u] = valid ? ldcg(p.rt + rb + bb[u]) : 0;
        }
        const bool wd = i0 == 0 && lane < j;
        off[kPgU] = wd ? S.off[lane] : 0;
        lo[kPgU] = 0;
        hi[kPgU] = wd ? S.n[lane] : 0;
        key[kPgU] = i;
        for (;;) {
            int t[kPgU + 1];
            bool any = false;
#pragma unroll
            for (int u = 0; u <= kPgU; ++u) {
                t[u] = 0;
                if (lo[u] < hi[u]) {
                    t[u] = ldcg(p.ot + off[u] + ((lo[u] + hi[u]) >> 1));
                    any = true;
                }
            }
            if (!any) break;
#pragma unroll
            for (int u = 0; u <= kPgU; ++u)
                if (lo[u] < hi[u]) {
                    const int mid = (lo[u] + hi[u]) >> 1;
                    if (t[u] < key[u])
                        lo[u] = mid + 1;
                    else
                        hi[u] = mid;
                }
        }
        if (wd) {
            const int q = lo[kPgU];
            if (q < S.n[lane] && ldcg(p.ot + off[kPgU] + q) == i) {
                S.dis[lane] = ldcg(p.ow + off[kPgU] + q);
            } else {  // the reference stops on this (something error2)
                S.dis[lane] = 0u;
                atomicOr(&p.ctl->flags, kPgErrRows);
            }
        }
        __syncwarp();  // the weights before the folds
#pragma unroll
        for (int u = 0; u < kPgU; ++u) {
            const int it = i0 + u * 32 + lane;
            if (it >= items) continue;
            const int q0 = qq[u], b = bb[u], an = S.n[q0], tb = key[u], lb = lo[u];
            const long long aoff = off[u];
            const int q = lb + ldcg(kbs + b);
            int ins = -1;
            if (q < an && ldcg(p.ot + aoff + q) == tb) {
                p.ow[aoff + q] = Rule::fold_hit(ldcg(p.ow + aoff + q), ldcg(p.rw + rb + b), S.dis[q0], p.keep);
            } else {  // after the row's pairs with this target (fewer than this pair's rank)
                ins = lb;
                while (ins < an && ldcg(p.ot + aoff + ins) == tb) ++ins;
                atomicAdd(&S.nnew[q0], 1);
            }
            insp[it] = ins;
        }
    }
    __syncwarp();
    for (int q0 = 0; q0 < j && nrm > 0; ++q0) {
        const int nk = S.nnew[q0];
        if (nk == 0) continue;  // every pair folded into an existing one, in place
        const int r = S.r[q0];
        const long long aoff = S.off[q0];
        const int an = S.n[q0];
        const unsigned dis = S.dis[q0];
        unsigned long long nb = 0;
        if (lane == 0) nb = atomicAdd(&p.ctl->out_top, (unsigned long long)(an + nk));
        nb = __shfl_sync(kFull, nb, 0);
        if (nb + (unsigned long long)(an + nk) > p.out_cap) {
            if (lane == 0) atomicOr(&p.ctl->flags, kPgErrPool);
            return;
        }
        const long long nbo = (long long)nb;
        int s0 = 0, last = 0;
        for (int b0 = 0; b0 < nrm; b0 += 32) {
            const int b = b0 + lane;
            const int ins = b < nrm ? ldcg(insp + q0 * nrm + b) : -1;
            const unsigned nwm = __ballot_sync(kFull, ins >= 0);
            const unsigned below = nwm & ((1u << lane) - 1u);
            const int pl = below ? 31 - __clz(below) : 0;
            const int pin = __shfl_sync(kFull, ins, pl);
            if (ins >= 0) {  // a new pair after the row's segment before it
                const int s = s0 + __popc(below);
                const int prev = below ? pin : last;
                pg_emit(p, par, 0, aoff + prev, nbo + prev + s, ins - prev);
                p.ot[nbo + ins + s] = ldcg(p.rt + rb + b);
                p.ow[nbo + ins + s] = Rule::fold_new(ldcg(p.rw + rb + b), dis, p.keep);
            }
            if (nwm) last = __shfl_sync(kFull, ins, 31 - __clz(nwm));
            s0 += __popc(nwm);
        }
        if (lane == 0) {
            pg_emit(p, par, 0, aoff + last, nbo + last + nk, an - last);
            p.out_off[r] = nbo;
            p.out_n[r] = an + nk;
        }
        __syncwarp();
    }
    if (lane == 0) {
        p.out_n[i] = kn;
        p.rec_off[i] = (long long)rb;
        p.rec_n[i] = nrm;
    }
}

// The queued copies of this round, one task per warp at a time.
__device__ __forceinline__ void pg_copy(const PgParams& p, int par, int gwarp, int nwarps, int lane) {
    const unsigned long long nt = min(ldcg(&p.ctl->task_top[par]), p.task_cap);
    for (unsigned long long t = (unsigned long long)gwarp; t < nt; t += (unsigned long long)nwarps) {
        const PgTask* tk = p.task + t;
        const long long src = ldl(&tk->src), dst = ldl(&tk->dst);
        const int len = ldcg(&tk->len), kind = ldcg(&tk->kind);
        // a task's source and destination never overlap: each lane loads its share of 256
        // entries before it stores any
        constexpr int kU = 8;
        for (int x0 = 0; x0 < len; x0 += 32 * kU) {
            if (kind == 0) {
                int tv[kU];
                unsigned wv[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int x = x0 + u * 32 + lane;
                    tv[u] = x < len ? ldcg(p.ot + src + x) : 0;
                    wv[u] = x < len ? ldcg(p.ow + src + x) : 0u;
                }
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int x = x0 + u * 32 + lane;
                    if (x < len) {
                        p.ot[dst + x] = tv[u];
                        p.ow[dst + x] = wv[u];
                    }
                }
            } else {
                int sv[kU];
                unsigned char av[kU];
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int x = x0 + u * 32 + lane;
                    sv[u] = x < len ? ldcg(p.is + src + x) : 0;
                    av[u] = x < len ? ldb(p.ia + src + x) : (unsigned char)0;
                }
#pragma unroll
                for (int u = 0; u < kU; ++u) {
                    const int x = x0 + u * 32 + lane;
                    if (x < len) {
                        p.is[dst + x] = sv[u];
                        p.ia[dst + x] = av[u];
                    }
                }
            }
        }
    }
}

// Position index -> (round k, vertex i).
__device__ __forceinline__ void pg_at(const PgParams& p, unsigned pos, int& k, int& i) {
    const unsigned q = pos / (unsigned)p.V;
    k = p.kfirst + (int)q;
    i = (int)(pos - q * (unsigned)p.V);
}

template <typename Rule>
__global__ void __launch_bounds__(kPgThreads, 3) prune_rounds(const PgParams p) {
    __shared__ PgRoots s_roots[kPgWarps];
    PgRoots& S = s_roots[threadIdx.x >> 5];
    PgCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gwarp = (int)(gtid >> 5), nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    unsigned long long tmark = globaltimer_ns();
    for (int guard = 0; guard < p.max_rounds; ++guard) {
        const unsigned pos = ldcg(&ctl->pos);
        const int round = ldcg(&ctl->round);
        const int par = round & 1;
        // Warp w owns the window's positions w, w + nwarps, ...; its lanes take up to 32 of
        // them at once.  A lane handles a position that only decides (reads its in-row and
        // out-row, writes nothing) by itself; the warp handles the ones that prune, one at a
        // time.
        // plan and reserve
        for (int b0 = 0; gwarp + b0 * nwarps < p.span; b0 += 32) {
            const int c = gwarp + (b0 + lane) * nwarps;
            const unsigned q = pos + (unsigned)c;
            const bool act = c < p.span && q < p.npos;
            int k = 0, i = 0;
            if (act) pg_at(p, q, k, i);
            const bool done = act && ldcg(p.pk + i) >= k;
            const bool heavy = act && !done && pg_prunes(p, i, k);
            if (done) p.slot_rn[c] = -1;
            if (act && !done && !heavy) {
                int* Rw = p.slot_r + (size_t)c * kPgSlotR;
                Rw[0] = p.V + i;
                Rw[1] = i;
                p.slot_rn[c] = 2;
                p.slot_woff[c] = 0;
                p.slot_wn[c] = 0;
                const unsigned long long key = pg_key(round, q);
                atomicMax(p.resA + p.V + i, key);
                atomicMax(p.resA + i, key);
            }
            unsigned hm = __ballot_sync(kFull, heavy);
            while (hm) {
                const int l = __ffs(hm) - 1;
                hm &= hm - 1u;
                const unsigned ql = __shfl_sync(kFull, q, l);
                const int il = __shfl_sync(kFull, i, l), kl = __shfl_sync(kFull, k, l);
                pg_plan<Rule>(p, ql, il, kl, gwarp + (b0 + l) * nwarps, round, lane, S);
            }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 0);
        // check: a position passes when no earlier position touches a row it writes or
        // writes a row it reads.  A position with an earlier writer of a row it reads may see
        // its plan change before it commits (whether that writer commits in this round or a
        // later one), and so may the rows it will touch: nothing after the first such position
        // commits in this round.
        for (int b0 = 0; gwarp + b0 * nwarps < p.span; b0 += 32) {
            const int c = gwarp + (b0 + lane) * nwarps;
            const unsigned q = pos + (unsigned)c;
            const bool act = c < p.span && q < p.npos;
            const int rn = act ? ldcg(p.slot_rn + c) : -1;
            const int wn = rn >= 0 ? ldcg(p.slot_wn + c) : 0;
            const bool light = rn == 2 && wn == 0;  // a decision: rows V + i and i read
            if (light) {
                int k, i;
                pg_at(p, q, k, i);
                const unsigned long long key = pg_key(round, q);
                const bool rok = ldcg(p.resW + p.V + i) <= key && ldcg(p.resW + i) <= key;
                p.slot_pass[c] = rok ? 1 : 0;
                if (!rok) atomicMin(&ctl->dmin, q);
            }
            unsigned hm = __ballot_sync(kFull, rn >= 0 && !light);
            while (hm) {
                const int l = __ffs(hm) - 1;
                hm &= hm - 1u;
                const int cl = gwarp + (b0 + l) * nwarps;
                const unsigned long long key = pg_key(round, pos + (unsigned)cl);
                const int rnl = __shfl_sync(kFull, rn, l), wnl = __shfl_sync(kFull, wn, l);
                const long long woff = ldl(p.slot_woff + cl);
                bool wok = true, rok = true;
                for (int x = lane; x < wnl; x += 32) wok = wok && ldcg(p.resA + ldcg(p.wscr + woff + x)) == key;
                if (lane < rnl) rok = ldcg(p.resW + ldcg(p.slot_r + (size_t)cl * kPgSlotR + lane)) <= key;
                wok = __all_sync(kFull, wok);
                rok = __all_sync(kFull, rok);
                if (lane == 0) {
                    p.slot_pass[cl] = (wok && rok) ? 1 : 0;
                    if (!rok) atomicMin(&ctl->dmin, pos + (unsigned)cl);
                }
            }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 1);
        // commit; the first position left pending starts the next window
        const unsigned dmin = ldcg(&ctl->dmin);
        if (gtid == 0 && dmin < p.npos) atomicMin(&ctl->nextpos, dmin);
        if (!(ldcg(flags) & (kPgErrPool | kPgErrRows))) {
            for (int b0 = 0; gwarp + b0 * nwarps < p.span; b0 += 32) {
                const int c = gwarp + (b0 + lane) * nwarps;
                const unsigned q = pos + (unsigned)c;
                const int rn = (c < p.span && q < p.npos && q <= dmin) ? ldcg(p.slot_rn + c) : -1;
                bool heavy = false;
                int k = 0, i = 0;
                if (rn >= 0) {
                    if (!ldb(p.slot_pass + c)) {
                        atomicMin(&ctl->nextpos, q);
                    } else {
                        pg_at(p, q, k, i);
                        // purn-sssp skips a vertex whose live in-degree is 0 or above k and
                        // visits the rest (src/purn-sssp.cpp:142-150), so one that went negative
                        // (two pairs with one target each kill i's in-entry) is visited and never
                        // pruned
                        const int d = ldcg(p.indeg + i);
                        const bool visit = d != 0 && d <= k;
                        heavy = visit && d > 0 && ldcg(p.out_n + i) > 0;
                        if (!heavy) p.pk[i] = visit ? p.klast : k;
                    }
                }
                unsigned hm = __ballot_sync(kFull, heavy);
                while (hm) {
                    const int l = __ffs(hm) - 1;
                    hm &= hm - 1u;
                    const int il = __shfl_sync(kFull, i, l), kl = __shfl_sync(kFull, k, l);
                    pg_visit<Rule>(p, il, kl, gwarp + (b0 + l) * nwarps, par, lane, S);
                    if (lane == 0) {
                        p.vk[il] = kl;
                        p.pk[il] = p.klast;
                    }
                }
            }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 2);
        // the queued copies; the next window from the first pending position, past the
        // positions already done behind it (a bounded look)
        pg_copy(p, par, gwarp, nwarps, lane);
        if (gtid < 32) {
            unsigned q = ldcg(&ctl->nextpos);
            for (int look = 0; look < 64 && q < p.npos; ++look) {
                const unsigned qq = q + (unsigned)lane;
                bool d = true;
                if (qq < p.npos) {
                    int k, i;
                    pg_at(p, qq, k, i);
                    d = ldcg(p.pk + i) >= k;
                }
                const unsigned m = __ballot_sync(kFull, d);
                if (m != kFull) {
                    q += (unsigned)(__ffs(~m) - 1);
                    break;
                }
                q += 32u;
            }
            q = min(q, p.npos);
            if (lane == 0) {
                ctl->pos = q;
                ctl->dmin = p.npos;
                ctl->nextpos = min(q + (unsigned)p.span, p.npos);
                ctl->round = round + 1;
                ctl->wscr_top = 0ull;
                ctl->mscr_top = 0ull;
                ctl->task_top[par ^ 1] = 0ull;
                if (q >= p.npos) ctl->finished = 1;
            }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 3);
        if (ldcg(&ctl->finished) || (ldcg(flags) & (kPgErrPool | kPgErrRows))) return;
    }
    if (gtid == 0) atomicOr(flags, C2G_FLAG_ITER_CAP);
}

// Rows listed by index, flat: row x's entries (off[x], n[x]) copied to base[x].
__global__ void pg_gather_rows(const long long* __restrict__ off, const int* __restrict__ n,
                               const long long* __restrict__ base, int rows, const int* __restrict__ t,
                               const unsigned* __restrict__ w, int* __restrict__ t_out, unsigned* __restrict__ w_out) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int v = warp; v < rows; v += nwarps) {
        const long long o = off[v], b = base[v];
        for (int k = lane; k < n[v]; k += 32) {
            t_out[b + k] = t[o + k];
            w_out[b + k] = w[o + k];
        }
    }
}

struct DevBuf {
    std::vector<void*> ptrs;
    ~DevBuf() {
        for (void* q : ptrs) cudaFree(q);
    }
    template <typename T>
    cudaError_t get(T** p, size_t n) {
        void* q = nullptr;
        const cudaError_t e = cudaMalloc(&q, sizeof(T) * (n ? n : 1));
        if (e == cudaSuccess) ptrs.push_back(q);
        *p = static_cast<T*>(q);
        return e;
    }
};

// Write n 4-byte elements of device memory to a file through a pinned staging buffer.
static int put_device_array(const std::string& path, const void* dev, size_t n, void* stage, size_t stage_n) {
    FILE* fp = fopen(path.c_str(), "wb");
    if (!fp) return fail(C2G_ERR_IO, "cannot create %s", path.c_str());
    for (size_t x = 0; x < n; x += stage_n) {
        const size_t k = std::min(stage_n, n - x);
        const cudaError_t ce = cudaMemcpy(stage, static_cast<const char*>(dev) + 4 * x, 4 * k, cudaMemcpyDeviceToHost);
        if (ce != cudaSuccess || fwrite(stage, 4, k, fp) != k) {
            fclose(fp);
            return ce != cudaSuccess ? fail(C2G_ERR_CUDA, "%s", cudaGetErrorString(ce))
                                     : fail(C2G_ERR_IO, "short write on %s", path.c_str());
        }
    }
    if (fclose(fp) != 0) return fail(C2G_ERR_IO, "short write on %s", path.c_str());
    return C2G_OK;
}

// One device pruning of dir's origin/ graph into dir/ppr/ (purn-ppr) or dir/sssp/
// (purn-sssp, with the record->vertex sidecar hvmap.bin).
template <typename Rule, typename W>
static int prune_device_dir(const std::string& dir, double keep, int device, float* ms, int* rounds,
                            int64_t* phase_ns) {
    constexpr bool kSssp = std::is_same<Rule, PgSssp>::value;
    int32_t V = 0;
    std::vector<int32_t> orow, ot, irow, is;
    std::vector<W> ow;
    int rc = prune_initial_rows<W>(dir, V, orow, ot, ow, irow, is);
    if (rc) return rc;
    const int kfirst = kSssp ? 1 : PgPpr::kMaxRoots, klast = Rule::kMaxRoots;
    const unsigned long long npos = (unsigned long long)(klast - kfirst + 1) * (unsigned long long)V;
    if (npos >= (1ull << 32)) return fail(C2G_ERR_RANGE, "pruner: %d vertices is too many for the device pruner", V);
    int prev = -1;
    cudaGetDevice(&prev);
    struct Restore {
        int d;
        ~Restore() {
            if (d >= 0) cudaSetDevice(d);
        }
    } restore{prev};
    C2G_CUDA(cudaSetDevice(device));
    int coop = 0, sms = 0, per_sm = 0;
    C2G_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, device));
    C2G_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device));
    if (!coop) return fail(C2G_ERR_UNSUPPORTED, "device lacks cooperative launch");
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prune_rounds<Rule>, kPgThreads, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "pruner kernel cannot be resident");
    const size_t E0 = ot.size(), I0 = is.size();
    // Window (measured at R-MAT scale 22): a wider one takes fewer rounds but more plan and
    // check work per round.  purn-ppr: 3,072 positions, 759 ms (1,024: 844; 2,048: 773;
    // 4,096: 802; 8,192: 914; 16,384: 1,042).  purn-sssp's positions are mostly decisions (a
    // vertex whose in-degree exceeds the round's bound), so its window is wider: 32,768,
    // 1,454 ms (16,384: 1,542; 24,576: 1,470; 65,536: 1,571).
    const int span = std::max(1, std::min(V, kSssp ? 32768 : 3072));
    // Pools: a row that gains entries takes a fresh block, so a pool holds every version of
    // its rows.  At R-MAT scale 20 / 22 purn-ppr's blocks add up to about 21 / 29 times the
    // original out-pairs and 22 / 33 times the original in-entries; give each 64 times,
    // within 60% of the free memory.
    size_t free_b = 0, total_b = 0;
    C2G_CUDA(cudaMemGetInfo(&free_b, &total_b));
    size_t out_cap = E0 * 64 + (1u << 20), in_cap_pool = I0 * 64 + (1u << 20);
    const double want = 8.0 * (double)out_cap + 5.0 * (double)in_cap_pool, room = 0.6 * (double)free_b;
    if (want > room) {
        out_cap = (size_t)((double)out_cap * room / want);
        in_cap_pool = (size_t)((double)in_cap_pool * room / want);
    }
    if (out_cap < E0 || in_cap_pool < I0) return fail(C2G_ERR_OOM, "pruner: not enough device memory for the row pools");
    const size_t rec_cap = E0 * 6 + (1u << 20);
    const size_t wscr_cap = E0 * 8 + (size_t)span * 64;
    const size_t mscr_cap = E0 * 8 + (1u << 20);
    const size_t task_cap = (size_t)1 << 22;
    DevBuf db;
    PgParams p;
    std::memset(&p, 0, sizeof(p));
    p.V = V;
    p.kfirst = kfirst;
    p.klast = klast;
    p.npos = (unsigned)npos;
    p.keep = keep;
    p.span = span;
    cudaError_t e = cudaSuccess;
    if (e == cudaSuccess) e = db.get(&p.out_off, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.out_n, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.ot, out_cap);
    if (e == cudaSuccess) e = db.get(&p.ow, out_cap);
    if (e == cudaSuccess) e = db.get(&p.in_off, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.in_n, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.is, in_cap_pool);
    if (e == cudaSuccess) e = db.get(&p.ia, in_cap_pool);
    if (e == cudaSuccess) e = db.get(&p.indeg, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.pk, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.vk, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.rec_off, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.rec_n, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.rt, rec_cap);
    if (e == cudaSuccess) e = db.get(&p.rw, rec_cap);
    if (e == cudaSuccess) e = db.get(&p.rmiss, rec_cap);
    if (e == cudaSuccess) e = db.get(&p.resA, 2 * (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.resW, 2 * (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.slot_r, (size_t)span * kPgSlotR);
    if (e == cudaSuccess) e = db.get(&p.slot_rn, (size_t)span);
    if (e == cudaSuccess) e = db.get(&p.slot_woff, (size_t)span);
    if (e == cudaSuccess) e = db.get(&p.slot_wn, (size_t)span);
    if (e == cudaSuccess) e = db.get(&p.slot_pass, (size_t)span);
    if (e == cudaSuccess) e = db.get(&p.wscr, wscr_cap);
    if (e == cudaSuccess) e = db.get(&p.mscr, mscr_cap);
    if (e == cudaSuccess) e = db.get(&p.task, task_cap);
    if (e == cudaSuccess) e = db.get(&p.ctl, 1);
    C2G_CUDA(e);
    p.out_cap = out_cap;
    p.in_pool_cap = in_cap_pool;
    p.rec_cap = rec_cap;
    p.wscr_cap = wscr_cap;
    p.mscr_cap = mscr_cap;
    p.task_cap = task_cap;
    p.barrier_ns = 20000000000ull;
    p.max_rounds = (int)std::min<unsigned long long>(npos + 16, 0x7fffffffull);
    {
        std::vector<long long> oo((size_t)V), io((size_t)V);
        std::vector<int> on((size_t)V), in_n((size_t)V), pk0((size_t)V, kfirst - 1);
        for (int32_t v = 0; v < V; ++v) {
            oo[v] = orow[v];
            on[v] = orow[v + 1] - orow[v];
            io[v] = irow[v];
            in_n[v] = irow[v + 1] - irow[v];
        }
        std::vector<unsigned char> alive(I0, 1);
        PgCtl c;
        std::memset(&c, 0, sizeof(c));
        c.out_top = E0;
        c.in_top = I0;
        c.pos = 0;
        c.dmin = p.npos;
        c.nextpos = std::min<unsigned>((unsigned)span, p.npos);
        c.round = 1;
        if (E0) {
            C2G_CUDA(cudaMemcpy(p.ot, ot.data(), sizeof(int32_t) * E0, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.ow, ow.data(), 4 * E0, cudaMemcpyHostToDevice));
        }
        if (I0) {
            C2G_CUDA(cudaMemcpy(p.is, is.data(), sizeof(int32_t) * I0, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.ia, alive.data(), I0, cudaMemcpyHostToDevice));
        }
        if (V > 0) {
            C2G_CUDA(cudaMemcpy(p.out_off, oo.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.out_n, on.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.in_off, io.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.in_n, in_n.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.indeg, in_n.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.pk, pk0.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
        }
        C2G_CUDA(cudaMemset(p.vk, 0, sizeof(int) * (size_t)V));
        C2G_CUDA(cudaMemset(p.rec_n, 0, sizeof(int) * (size_t)V));
        C2G_CUDA(cudaMemset(p.rec_off, 0, sizeof(long long) * (size_t)V));
        C2G_CUDA(cudaMemset(p.resA, 0, sizeof(unsigned long long) * 2 * (size_t)V));
        C2G_CUDA(cudaMemset(p.resW, 0, sizeof(unsigned long long) * 2 * (size_t)V));
        C2G_CUDA(cudaMemcpy(p.ctl, &c, sizeof(c), cudaMemcpyHostToDevice));
    }
    std::vector<int32_t>().swap(ot);
    std::vector<W>().swap(ow);
    std::vector<int32_t>().swap(is);
    cudaEvent_t e0, e1;
    C2G_CUDA(cudaEventCreate(&e0));
    C2G_CUDA(cudaEventCreate(&e1));
    void* args[] = {&p};
    cudaEventRecord(e0);
    e = V > 0 ? cudaLaunchCooperativeKernel((const void*)prune_rounds<Rule>, dim3(per_sm * sms), dim3(kPgThreads), args,
                                            0, nullptr)
              : cudaSuccess;
    cudaEventRecord(e1);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    C2G_CUDA(e);
    PgCtl c;
    C2G_CUDA(cudaMemcpy(&c, p.ctl, sizeof(c), cudaMemcpyDeviceToHost));
    if (ms) *ms = t;
    if (rounds) *rounds = c.round - 1;
    if (phase_ns)
        for (int k = 0; k < 4; ++k) phase_ns[k] = (int64_t)c.phase_ns[k];
    if (c.flags & kPgErrPool) return fail(C2G_ERR_OVERFLOW, "pruner: a row pool ran out");
    if (c.flags & kPgErrRows) return fail(C2G_ERR_FORMAT, "pruner: in-row and out-rows disagree");
    if (c.flags & (C2G_FLAG_BARRIER_TIMEOUT | C2G_FLAG_ITER_CAP) || (V > 0 && !c.finished))
        return fail(C2G_ERR_TIMEOUT, "pruner: rounds did not finish (flags %d)", c.flags);
    // Records: purn-ppr has one per vertex in id order (empty when it is not pruned);
    // purn-sssp one per pruned vertex in visiting order, (round, id), with the sidecar.
    std::vector<int> on((size_t)V), rn((size_t)V), vk((size_t)V);
    std::vector<long long> roff((size_t)V);
    if (V > 0) {
        C2G_CUDA(cudaMemcpy(on.data(), p.out_n, sizeof(int) * (size_t)V, cudaMemcpyDeviceToHost));
        C2G_CUDA(cudaMemcpy(rn.data(), p.rec_n, sizeof(int) * (size_t)V, cudaMemcpyDeviceToHost));
        C2G_CUDA(cudaMemcpy(vk.data(), p.vk, sizeof(int) * (size_t)V, cudaMemcpyDeviceToHost));
        C2G_CUDA(cudaMemcpy(roff.data(), p.rec_off, sizeof(long long) * (size_t)V, cudaMemcpyDeviceToHost));
    }
    std::vector<int32_t> order;
    if (kSssp) {
        std::vector<int32_t> cnt((size_t)klast + 2, 0);
        for (int32_t v = 0; v < V; ++v)
            if (vk[v] > 0) ++cnt[(size_t)vk[v] + 1];
        for (int k = 1; k <= klast + 1; ++k) cnt[k] += cnt[k - 1];
        order.resize((size_t)cnt[(size_t)klast + 1]);
        for (int32_t v = 0; v < V; ++v)
            if (vk[v] > 0) order[(size_t)cnt[(size_t)vk[v]]++] = v;
    } else {
        order.resize((size_t)V);
        for (int32_t v = 0; v < V; ++v) order[v] = v;
    }
    const size_t H = order.size();
    std::vector<int32_t> pv((size_t)V + 1, 0), hv(H + 1, 0);
    std::vector<long long> ob((size_t)V), hoff(H), hb(H);
    std::vector<int> hn(H);
    for (int32_t v = 0; v < V; ++v) {
        ob[v] = pv[v];
        pv[v + 1] = pv[v] + on[v];
    }
    for (size_t x = 0; x < H; ++x) {
        hoff[x] = roff[order[x]];
        hn[x] = rn[order[x]];
        hb[x] = hv[x];
        hv[x + 1] = hv[x] + hn[x];
    }
    const size_t E = (size_t)pv[V], HE = (size_t)hv[H];
    DevBuf tmp;
    long long *dob = nullptr, *dhoff = nullptr, *dhb = nullptr;
    int *dhn = nullptr, *dpe = nullptr, *dhe = nullptr;
    unsigned *dpw = nullptr, *dhw = nullptr;
    e = tmp.get(&dob, (size_t)V);
    if (e == cudaSuccess) e = tmp.get(&dhoff, H);
    if (e == cudaSuccess) e = tmp.get(&dhb, H);
    if (e == cudaSuccess) e = tmp.get(&dhn, H);
    if (e == cudaSuccess) e = tmp.get(&dpe, E);
    if (e == cudaSuccess) e = tmp.get(&dpw, E);
    if (e == cudaSuccess) e = tmp.get(&dhe, HE);
    if (e == cudaSuccess) e = tmp.get(&dhw, HE);
    C2G_CUDA(e);
    if (V > 0) C2G_CUDA(cudaMemcpy(dob, ob.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
    if (H > 0) {
        C2G_CUDA(cudaMemcpy(dhoff, hoff.data(), sizeof(long long) * H, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(dhb, hb.data(), sizeof(long long) * H, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(dhn, hn.data(), sizeof(int) * H, cudaMemcpyHostToDevice));
    }
    if (V > 0) pg_gather_rows<<<sms * 8, 256>>>(p.out_off, p.out_n, dob, V, p.ot, p.ow, dpe, dpw);
    if (H > 0) pg_gather_rows<<<sms * 8, 256>>>(dhoff, dhn, dhb, (int)H, p.rt, p.rw, dhe, dhw);
    C2G_CUDA(cudaGetLastError());
    C2G_CUDA(cudaDeviceSynchronize());
    const size_t stage_n = (size_t)1 << 24;
    void* stage = nullptr;
    C2G_CUDA(cudaMallocHost(&stage, 4 * stage_n));
    struct FreeHost {
        void* q;
        ~FreeHost() { cudaFreeHost(q); }
    } free_stage{stage};
    const std::string sub = kSssp ? "sssp" : "ppr";
    const std::string s = dir + "/" + sub + "/";
    if ((rc = make_dir(dir + "/" + sub))) return rc;
    if ((rc = write_array4(s + "hvlist.bin", hv.data(), hv.size()))) return rc;
    if ((rc = put_device_array(s + "helist.bin", dhe, HE, stage, stage_n))) return rc;
    if ((rc = put_device_array(s + "hwlist.bin", dhw, HE, stage, stage_n))) return rc;
    if (kSssp && (rc = write_array4(s + "hvmap.bin", order.data(), order.size()))) return rc;
    if ((rc = write_array4(s + "vlist.bin", pv.data(), pv.size()))) return rc;
    if ((rc = put_device_array(s + "elist.bin", dpe, E, stage, stage_n))) return rc;
    if ((rc = put_device_array(s + "wlist.bin", dpw, E, stage, stage_n))) return rc;
    return C2G_OK;
}

}  // namespace c2g

extern "C" int c2g_prune_ppr_device(const char* dir, double alpha, int device, float* ms, int32_t* rounds,
                                    int64_t* phase_ns) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "prune: dir is NULL");
    if (!(alpha > 0.0 && alpha < 1.0)) return c2g::fail(C2G_ERR_ARG, "prune: alpha must be in (0, 1)");
    return c2g::prune_device_dir<c2g::PgPpr, float>(dir, 1.0 - alpha, device, ms, rounds, phase_ns);
}

extern "C" int c2g_prune_sssp_device(const char* dir, int device, float* ms, int32_t* rounds, int64_t* phase_ns) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "prune: dir is NULL");
    return c2g::prune_device_dir<c2g::PgSssp, int32_t>(dir, 0.0, device, ms, rounds, phase_ns);
}
