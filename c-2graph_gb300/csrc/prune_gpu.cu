// purn-ppr on the GPU (src/purn-ppr.cpp:63-344), writing the same bytes as the host pass
// (prune.cpp) and the reference.
//
// The reference visits every vertex once in id order; a visit with live in-degree in
// [1, 5] and out-edges moves each out-edge i -> v that every live in-neighbour ("root")
// of i but at most one already has into the roots' rows, with folded weights, and
// records it.  A visit reads its in-row, its out-row and its roots' out-rows, and writes
// its out-row, its roots' out-rows and the in-rows of the targets it moves, so the order
// matters only between visits that share rows.  The device pruner runs the same visits in
// rounds of a speculative schedule (deterministic reservations): every unvisited vertex of
// a window plans its visit on the current state (the rows it reads and would write, and
// which out-edges move) and reserves those rows under its id; it commits when no earlier
// candidate of the window writes a row it reads or touches a row it writes, unless an
// earlier candidate that failed had a row it reads written in this round (its plan may
// change), past which nothing commits.  The first unvisited vertex always commits, so every
// round makes progress.  The schedule is the one orc_prune_ppr_speculative checks on the
// CPU.
//
// Committed visits touch disjoint rows and run in parallel, one warp each, with the
// reference's steps: roots in in-row order; the out-row split into kept pairs (compacted
// in place) and moved pairs (the record); each moved target's in-row gains the roots that
// lack the target (a revived entry, or an inserted one) and loses i; the moved pairs merge
// into each root's sorted row, a pair with a target the row has adding (w * keep) * w' to
// the weight (double, rounded to float), a new target inserted with that weight.  Updates
// of existing entries are made in place.  A row that gains entries moves to a new block of
// its pool (bump allocation): the visit writes the new entries there and queues the old
// row's segments between them as copy tasks of at most kPgTask elements, which the whole
// grid runs after the commit phase.  So the copying of long rows (hubs are the roots of
// many pruned vertices) is spread over every SM instead of one warp.
#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/c2graph.h"
#include "device_common.cuh"
#include "host_io.h"
#include "internal.h"

namespace c2g {

int prune_ppr_initial_rows(const std::string& dir, int32_t& V, std::vector<int32_t>& orow, std::vector<int32_t>& ot,
                           std::vector<float>& ow, std::vector<int32_t>& irow, std::vector<int32_t>& is);

constexpr int kPgThreads = 256;
constexpr int kPgMaxRoots = 5;  // the in-degree bound of purn-ppr (src/purn-ppr.cpp:146-152)
constexpr int kPgMaxR = 2 + kPgMaxRoots;  // rows a visit reads: its in-row, its out-row, its roots' out-rows
constexpr int kPgTask = 1024;             // elements per copy task
constexpr int kPgMoved = 0x100;           // plan code of an out-edge that moves (| the roots lacking it)

struct PgCtl {
    unsigned bar_count, bar_gen;  // GridBarrier
    int flags;
    int pos;    // the first unvisited vertex
    int dmin;   // this round: the first failed candidate whose reads a committer writes
    int round;
    int finished;
    int pad;
    unsigned long long out_top, in_top, rec_top, wscr_top;  // pool bump pointers
    unsigned long long task_top[2];                         // copy tasks, by round parity
    unsigned long long phase_ns[5];  // block 0's time in plan, check, disturb, commit, copy (waits included)
};

struct PgTask {
    long long src, dst;
    int len, kind;  // kind 0: out-row pairs (ot, ow); 1: in-row entries (is, ia)
};

struct PgParams {
    int V;
    double keep;
    int span;  // window: candidates pos .. pos + span - 1
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
    long long* rec_off;
    int* rec_n;
    int* rt;
    unsigned* rw;
    unsigned char* rmiss;  // per moved pair: the roots (bits, root order) without its target
    unsigned long long rec_cap;
    unsigned char* done;
    unsigned long long* resA;  // [2V] (round << 32) | ~id, the earliest candidate touching the row
    unsigned long long* resW;  // [2V] the same for writers
    int* wmark;                // [2V] round in which a committer writes the row
    int* slot_r;               // [span][kPgMaxR] rows read (out-row x is x, in-row x is V + x)
    int* slot_rn;              // rows read, -1: no candidate
    long long* slot_woff;      // plan block in wscr: rows written, then one code per out-edge
    int* slot_wn;
    unsigned char* slot_pass;
    int* wscr;
    unsigned long long wscr_cap;
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

__device__ __forceinline__ unsigned long long pg_key(int round, int i) {
    return ((unsigned long long)(unsigned)round << 32) | (unsigned long long)(~(unsigned)i);
}

// first index of [lo, n) of row `off` of `t` with t > key (upper) or t >= key (lower), or n
__device__ __forceinline__ int pg_search(const int* t, long long off, int lo, int n, int key, bool upper) {
    int hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int x = ldcg(t + off + mid);
        if (x < key || (upper && x == key))
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// A vertex's live roots in in-row order and their out-rows (registers; indexed only in
// unrolled loops).
struct PgRoots {
    int j;
    int r[kPgMaxRoots];
    long long off[kPgMaxRoots];
    int n[kPgMaxRoots];
};

template <typename T>
__device__ __forceinline__ T pg_pick(const T (&a)[kPgMaxRoots], int k) {
    T x = a[0];
#pragma unroll
    for (int q = 1; q < kPgMaxRoots; ++q)
        if (q == k) x = a[q];
    return x;
}

// The live roots of i (every lane gets them).  Returns their count (kPgMaxRoots + 1 means
// more than kPgMaxRoots; R.j keeps the first kPgMaxRoots).
__device__ __forceinline__ int pg_roots(const PgParams& p, int i, PgRoots& R, int lane) {
    const long long off = ldl(p.in_off + i);
    const int n = ldcg(p.in_n + i);
    int nr = 0;
#pragma unroll
    for (int q = 0; q < kPgMaxRoots; ++q) R.r[q] = 0;
    for (int b = 0; b < n && nr <= kPgMaxRoots; b += 32) {
        const int k = b + lane;
        const bool a = k < n && ldb(p.ia + off + k) != 0;
        const int s = k < n ? ldcg(p.is + off + k) : 0;
        unsigned m = __ballot_sync(kFull, a);
        while (m && nr <= kPgMaxRoots) {
            const int src = __shfl_sync(kFull, s, __ffs(m) - 1);
#pragma unroll
            for (int q = 0; q < kPgMaxRoots; ++q)
                if (q == nr) R.r[q] = src;
            ++nr;
            m &= m - 1u;
        }
    }
    R.j = min(nr, kPgMaxRoots);
#pragma unroll
    for (int q = 0; q < kPgMaxRoots; ++q) {
        R.off[q] = 0;
        R.n[q] = 0;
        if (q < R.j) {
            R.off[q] = ldl(p.out_off + R.r[q]);
            R.n[q] = ldcg(p.out_n + R.r[q]);
        }
    }
    return nr;
}

// Does the edge i -> v move (every root but at most one has v)?  miss: roots without v.
// Membership in a root's sorted row is the reference's monotone cursor test
// (src/purn-ppr.cpp:170-186) as a lower bound; the roots' searches run in lockstep.
__device__ __forceinline__ bool pg_moves(const PgParams& p, const PgRoots& R, int v, unsigned& miss) {
    miss = 0u;
    bool root = false;
#pragma unroll
    for (int k = 0; k < kPgMaxRoots; ++k) root |= k < R.j && R.r[k] == v;
    if (root) return false;  // a root keeps its edge
    int lo[kPgMaxRoots], hi[kPgMaxRoots];
#pragma unroll
    for (int k = 0; k < kPgMaxRoots; ++k) {
        lo[k] = 0;
        hi[k] = k < R.j ? R.n[k] : 0;
    }
    for (;;) {
        int t[kPgMaxRoots];
        bool any = false;
#pragma unroll
        for (int k = 0; k < kPgMaxRoots; ++k) {
            t[k] = 0;
            if (lo[k] < hi[k]) {
                t[k] = ldcg(p.ot + R.off[k] + ((lo[k] + hi[k]) >> 1));
                any = true;
            }
        }
        if (!any) break;
#pragma unroll
        for (int k = 0; k < kPgMaxRoots; ++k)
            if (lo[k] < hi[k]) {
                const int mid = (lo[k] + hi[k]) >> 1;
                if (t[k] < v)
                    lo[k] = mid + 1;
                else
                    hi[k] = mid;
            }
    }
    int cnt = 0;
#pragma unroll
    for (int k = 0; k < kPgMaxRoots; ++k) {
        if (k >= R.j) continue;
        if (lo[k] < R.n[k] && ldcg(p.ot + R.off[k] + lo[k]) == v)
            ++cnt;
        else
            miss |= 1u << k;
    }
    return cnt + 2 > R.j;
}

__device__ __forceinline__ bool pg_prunes(const PgParams& p, int i) {
    const int d = ldcg(p.indeg + i);
    return ldcg(p.out_n + i) > 0 && d > 0 && d <= kPgMaxRoots;
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

// Plan of candidate i (slot c): the rows it reads, the rows it would write, and per
// out-edge whether it moves; reserve the rows.  The plan block in wscr holds the written
// rows (at most on + 6) in [0, on + 8) and the out-edge codes in [on + 8, 2 on + 8); the
// commit reuses [on + 8, 7 on + 8) for the merges' scratch.
__device__ __forceinline__ void pg_plan(const PgParams& p, int i, int c, int round, int lane) {
    const int V = p.V;
    int* Rw = p.slot_r + (size_t)c * kPgMaxR;
    int rn = 2;
    if (lane == 0) {
        Rw[0] = V + i;
        Rw[1] = i;
    }
    long long woff = 0;
    int wn = 0;
    if (pg_prunes(p, i)) {
        PgRoots R;
        pg_roots(p, i, R, lane);
        const int j = R.j;
        if (lane == 0) {
#pragma unroll
            for (int k = 0; k < kPgMaxRoots; ++k)
                if (k < j) Rw[2 + k] = R.r[k];
        }
        rn = 2 + j;
        const long long off = ldl(p.out_off + i);
        const int on = ldcg(p.out_n + i);
        const unsigned long long need = 7ull * (unsigned long long)on + 8ull;
        unsigned long long wb = 0;
        if (lane == 0) wb = atomicAdd(&p.ctl->wscr_top, need);
        wb = __shfl_sync(kFull, wb, 0);
        if (wb + need > p.wscr_cap) {
            if (lane == 0) atomicOr(&p.ctl->flags, kPgErrPool);
        } else {
            woff = (long long)wb;
            int* code = p.wscr + woff + on + 8;
            for (int b = 0; b < on; b += 32) {
                const int e = b + lane;
                unsigned miss = 0u;
                const int v = e < on ? ldcg(p.ot + off + e) : 0;
                const bool mv = e < on && pg_moves(p, R, v, miss);
                if (e < on) code[e] = mv ? (int)(kPgMoved | miss) : 0;
                const unsigned m = __ballot_sync(kFull, mv);
                if (mv) p.wscr[woff + wn + __popc(m & ((1u << lane) - 1u))] = V + v;
                wn += __popc(m);
            }
            if (wn > 0) {  // it moves edges: its out-row and its roots' out-rows change
                if (lane == 0) {
                    p.wscr[woff + wn] = i;
#pragma unroll
                    for (int k = 0; k < kPgMaxRoots; ++k)
                        if (k < j) p.wscr[woff + wn + 1 + k] = R.r[k];
                }
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
    const unsigned long long key = pg_key(round, i);
    if (lane < rn) atomicMax(p.resA + Rw[lane], key);
    for (int k = lane; k < wn; k += 32) {
        const int r = p.wscr[woff + k];
        atomicMax(p.resA + r, key);
        atomicMax(p.resW + r, key);
    }
}

// v's in-row after the `cnt` moved pairs i -> v of a visit (one lane): every root in `miss`
// gets a live entry (revived, or inserted in source order) and counts in v's in-degree, and
// i's entry dies once per pair (src/purn-ppr.cpp:196-236).
__device__ __forceinline__ void pg_in_update(const PgParams& p, const PgRoots& R, int i, int v, unsigned miss,
                                             int cnt, int par) {
    const long long off = ldl(p.in_off + v);
    const int n = ldcg(p.in_n + v);
    // lockstep lower bounds: the missing roots (0 .. kPgMaxRoots - 1) and i (kPgMaxRoots)
    int lo[kPgMaxRoots + 1], hi[kPgMaxRoots + 1];
#pragma unroll
    for (int k = 0; k <= kPgMaxRoots; ++k) {
        const bool use = k == kPgMaxRoots || (k < R.j && ((miss >> k) & 1u));
        lo[k] = 0;
        hi[k] = use ? n : 0;
    }
    for (;;) {
        int t[kPgMaxRoots + 1];
        bool any = false;
#pragma unroll
        for (int k = 0; k <= kPgMaxRoots; ++k) {
            t[k] = 0;
            if (lo[k] < hi[k]) {
                t[k] = ldcg(p.is + off + ((lo[k] + hi[k]) >> 1));
                any = true;
            }
        }
        if (!any) break;
#pragma unroll
        for (int k = 0; k <= kPgMaxRoots; ++k)
            if (lo[k] < hi[k]) {
                const int mid = (lo[k] + hi[k]) >> 1;
                const int key = k < kPgMaxRoots ? R.r[k] : i;
                if (t[k] < key)
                    lo[k] = mid + 1;
                else
                    hi[k] = mid;
            }
    }
    const int qi = lo[kPgMaxRoots];
    if (qi >= n || ldcg(p.is + off + qi) != i) {
        atomicOr(&p.ctl->flags, kPgErrRows);
        return;
    }
    int inc = 0;
    unsigned ins = 0u;
#pragma unroll
    for (int k = 0; k < kPgMaxRoots; ++k) {
        if (!(k < R.j && ((miss >> k) & 1u))) continue;
        const int q = lo[k];
        if (q < n && ldcg(p.is + off + q) == R.r[k]) {
            if (!ldb(p.ia + off + q)) {
                p.ia[off + q] = 1;
                ++inc;
            }
        } else {
            ins |= 1u << k;
            ++inc;
        }
    }
    p.ia[off + qi] = 0;
    p.indeg[v] = ldcg(p.indeg + v) + inc - cnt;
    if (ins) {
        const int nins = __popc(ins);
        const unsigned long long nb = atomicAdd(&p.ctl->in_top, (unsigned long long)(n + nins));
        if (nb + (unsigned long long)(n + nins) > p.in_pool_cap) {
            atomicOr(&p.ctl->flags, kPgErrPool);
            return;
        }
        const long long nbo = (long long)nb;
        int s = 0, prev = 0;
#pragma unroll
        for (int k = 0; k < kPgMaxRoots; ++k) {
            if (!((ins >> k) & 1u)) continue;
            const int at = lo[k];  // roots ascend, so the insertion points do too
            pg_emit(p, par, 1, off + prev, nbo + prev + s, at - prev);
            p.is[nbo + at + s] = R.r[k];
            p.ia[nbo + at + s] = 1;
            prev = at;
            ++s;
        }
        pg_emit(p, par, 1, off + prev, nbo + prev + s, n - prev);
        p.in_off[v] = nbo;
        p.in_n[v] = n + nins;
    }
}

// A committed visit of vertex i (slot c; the plan's rows are unchanged since the plan).
__device__ __forceinline__ void pg_visit(const PgParams& p, int i, int c, int par, int lane) {
    PgRoots R;
    const int nr = pg_roots(p, i, R, lane);
    const int j = R.j;
    if (nr != ldcg(p.indeg + i) || nr > kPgMaxRoots) {  // the reference stops on this (something error2)
        if (lane == 0) atomicOr(&p.ctl->flags, kPgErrRows);
        return;
    }
    // lane k < j: the weight of root k -> i, its first pair with target i
    unsigned dis = 0u;
    if (lane < j) {
        const long long off = pg_pick(R.off, lane);
        const int n = pg_pick(R.n, lane);
        const int q = pg_search(p.ot, off, 0, n, i, false);
        if (q < n && ldcg(p.ot + off + q) == i)
            dis = ldcg(p.ow + off + q);
        else
            atomicOr(&p.ctl->flags, kPgErrRows);
    }
    const long long ooff = ldl(p.out_off + i);
    const int on = ldcg(p.out_n + i);
    const long long woff = ldl(p.slot_woff + c);
    const int wn = ldcg(p.slot_wn + c);
    const int nrm = wn > 0 ? wn - 1 - j : 0;
    int* code = p.wscr + woff + on + 8;
    unsigned long long rb = 0;
    if (nrm > 0) {
        if (lane == 0) rb = atomicAdd(&p.ctl->rec_top, (unsigned long long)nrm);
        rb = __shfl_sync(kFull, rb, 0);
        if (rb + (unsigned long long)nrm > p.rec_cap) {
            if (lane == 0) atomicOr(&p.ctl->flags, kPgErrPool);
            return;
        }
    }
    // split the out-row: moved pairs to the record (in order), kept ones compacted in place
    int nm = 0, kn = 0;
    for (int b = 0; b < on; b += 32) {
        const int e = b + lane;
        const bool valid = e < on;
        const int v = valid ? ldcg(p.ot + ooff + e) : 0;
        const unsigned w = valid ? ldcg(p.ow + ooff + e) : 0u;
        const int cd = valid ? ldcg(code + e) : 0;
        const bool mv = (cd & kPgMoved) != 0;
        const bool kp = valid && !mv;
        const unsigned mm = __ballot_sync(kFull, mv), mk = __ballot_sync(kFull, kp);
        const unsigned lt = (1u << lane) - 1u;
        if (mv) {
            const int x = nm + __popc(mm & lt);
            if (x < nrm) {
                p.rt[rb + x] = v;
                p.rw[rb + x] = w;
                p.rmiss[rb + x] = (unsigned char)(cd & 0xff);
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
        pg_in_update(p, R, i, v, ldb(p.rmiss + rb + b), cnt, par);
    }
    __syncwarp();
    // The moved pairs merge into every root's sorted row.  Pass 1 takes every (root, pair)
    // item at once: a pair whose target the row has (the k-th pair of a run of equal targets
    // goes with the row's k-th pair of that target, as the reference's two-cursor merge pairs
    // them) adds (w * keep) * w' to that pair in place, in double, rounded to float; a new
    // one gets its insertion point.  The codes' space holds each pair's rank in its run, then
    // the items' insertion points (-1: added in place).  Pass 2 moves each root's row that
    // gains pairs to a new block.
    int* kbs = code;
    int* insp = code + nrm;
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
    int nnew[kPgMaxRoots];
#pragma unroll
    for (int k = 0; k < kPgMaxRoots; ++k) nnew[k] = 0;
    const int items = j * nrm;
    for (int i0 = 0; i0 < items; i0 += 32) {
        const int it = i0 + lane;
        const bool valid = it < items;
        const int k = valid ? it / nrm : 0;
        const int b = valid ? it - k * nrm : 0;
        const double dk = (double)__uint_as_float((unsigned)__shfl_sync(kFull, (int)dis, k));
        int ins = -1;
        if (valid) {
            const long long aoff = pg_pick(R.off, k);
            const int an = pg_pick(R.n, k);
            const int tb = ldcg(p.rt + rb + b);
            const int lb = pg_search(p.ot, aoff, 0, an, tb, false);
            const int q = lb + ldcg(kbs + b);
            if (q < an && ldcg(p.ot + aoff + q) == tb) {
                const double f = __dmul_rn(__dmul_rn((double)__uint_as_float(ldcg(p.rw + rb + b)), p.keep), dk);
                p.ow[aoff + q] = __float_as_uint(
                    __double2float_rn(__dadd_rn((double)__uint_as_float(ldcg(p.ow + aoff + q)), f)));
            } else {  // after the row's pairs with this target (fewer than this pair's rank)
                ins = lb;
                while (ins < an && ldcg(p.ot + aoff + ins) == tb) ++ins;
            }
            insp[it] = ins;
        }
#pragma unroll
        for (int kk = 0; kk < kPgMaxRoots; ++kk) nnew[kk] += __popc(__ballot_sync(kFull, ins >= 0 && k == kk));
    }
    __syncwarp();
    for (int k = 0; k < j; ++k) {
        const int nk = pg_pick(nnew, k);
        if (nk == 0) continue;  // every pair added to an existing one, in place
        const int r = pg_pick(R.r, k);
        const long long aoff = pg_pick(R.off, k);
        const int an = pg_pick(R.n, k);
        const double dk = (double)__uint_as_float((unsigned)__shfl_sync(kFull, (int)dis, k));
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
            const int ins = b < nrm ? ldcg(insp + k * nrm + b) : -1;
            const unsigned nwm = __ballot_sync(kFull, ins >= 0);
            const unsigned below = nwm & ((1u << lane) - 1u);
            const int pl = below ? 31 - __clz(below) : 0;
            const int pin = __shfl_sync(kFull, ins, pl);
            if (ins >= 0) {  // a new pair: (w * keep) * w', to float, after the row's segment before it
                const int s = s0 + __popc(below);
                const int prev = below ? pin : last;
                pg_emit(p, par, 0, aoff + prev, nbo + prev + s, ins - prev);
                const double f = __dmul_rn(__dmul_rn((double)__uint_as_float(ldcg(p.rw + rb + b)), p.keep), dk);
                p.ot[nbo + ins + s] = ldcg(p.rt + rb + b);
                p.ow[nbo + ins + s] = __float_as_uint(__double2float_rn(f));
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

__global__ void __launch_bounds__(kPgThreads, 3) prune_ppr_rounds(const PgParams p) {
    PgCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gwarp = (int)(gtid >> 5), nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    unsigned long long tmark = globaltimer_ns();
    for (int guard = 0; guard < p.max_rounds; ++guard) {
        const int pos = ldcg(&ctl->pos), round = ldcg(&ctl->round);
        const int par = round & 1;
        // plan and reserve
        for (int c = gwarp; c < p.span; c += nwarps) {
            const int i = pos + c;
            if (i >= p.V) break;
            if (ldb(p.done + i)) {
                if (lane == 0) p.slot_rn[c] = -1;
                continue;
            }
            pg_plan(p, i, c, round, lane);
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 0);
        // check: the passers mark the rows they write
        for (int c = gwarp; c < p.span; c += nwarps) {
            const int i = pos + c;
            if (i >= p.V) break;
            const int rn = ldcg(p.slot_rn + c);
            if (rn < 0) continue;
            const unsigned long long key = pg_key(round, i);
            const long long woff = ldl(p.slot_woff + c);
            const int wn = ldcg(p.slot_wn + c);
            bool ok = true;
            for (int k = lane; k < wn; k += 32) ok = ok && ldcg(p.resA + ldcg(p.wscr + woff + k)) == key;
            if (lane < rn) ok = ok && ldcg(p.resW + ldcg(p.slot_r + (size_t)c * kPgMaxR + lane)) <= key;
            ok = __all_sync(kFull, ok);
            if (lane == 0) p.slot_pass[c] = ok ? 1 : 0;
            if (ok)
                for (int k = lane; k < wn; k += 32) p.wmark[ldcg(p.wscr + woff + k)] = round;
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 1);
        // a failed candidate whose reads a passer writes holds back the ones after it
        for (int c = gwarp; c < p.span; c += nwarps) {
            const int i = pos + c;
            if (i >= p.V) break;
            const int rn = ldcg(p.slot_rn + c);
            if (rn < 0 || ldb(p.slot_pass + c)) continue;
            const bool hit = lane < rn && ldcg(p.wmark + ldcg(p.slot_r + (size_t)c * kPgMaxR + lane)) == round;
            if (__any_sync(kFull, hit) && lane == 0) atomicMin(&ctl->dmin, i);
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 2);
        // commit
        const int dmin = ldcg(&ctl->dmin);
        if (!(ldcg(flags) & (kPgErrPool | kPgErrRows))) {
            for (int c = gwarp; c < p.span; c += nwarps) {
                const int i = pos + c;
                if (i >= p.V || i > dmin) break;
                if (ldcg(p.slot_rn + c) < 0 || !ldb(p.slot_pass + c)) continue;
                if (pg_prunes(p, i)) pg_visit(p, i, c, par, lane);
                if (lane == 0) p.done[i] = 1;
            }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 3);
        // the queued copies; the next window
        pg_copy(p, par, gwarp, nwarps, lane);
        if (gtid < 32) {
            int q = pos;
            for (;;) {
                const int k = q + lane;
                const bool d = k >= p.V || ldb(p.done + k);
                const unsigned m = __ballot_sync(kFull, d);
                if (m != kFull) {
                    q += __ffs(~m) - 1;
                    break;
                }
                q += 32;
                if (q >= p.V) break;
            }
            if (lane == 0) {
                ctl->pos = min(q, p.V);
                ctl->dmin = p.V;
                ctl->round = round + 1;
                ctl->wscr_top = 0ull;
                ctl->task_top[par ^ 1] = 0ull;
                if (q >= p.V) ctl->finished = 1;
            }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        phase_mark(ctl->phase_ns, tmark, 4);
        if (ldcg(&ctl->finished) || (ldcg(flags) & (kPgErrPool | kPgErrRows))) return;
    }
    if (gtid == 0) atomicOr(flags, C2G_FLAG_ITER_CAP);
}

// The final rows and records, flat: row r's pairs (or records) copied to base[r].
__global__ void pg_gather_rows(const long long* __restrict__ off, const int* __restrict__ n,
                               const long long* __restrict__ base, int V, const int* __restrict__ t,
                               const unsigned* __restrict__ w, int* __restrict__ t_out, unsigned* __restrict__ w_out) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int v = warp; v < V; v += nwarps) {
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

static int prune_ppr_device_dir(const std::string& dir, double keep, int device, float* ms, int* rounds,
                                int64_t* phase_ns) {
    int32_t V = 0;
    std::vector<int32_t> orow, ot, irow, is;
    std::vector<float> ow;
    int rc = prune_ppr_initial_rows(dir, V, orow, ot, ow, irow, is);
    if (rc) return rc;
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
    C2G_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, prune_ppr_rounds, kPgThreads, 0));
    if (per_sm < 1) return fail(C2G_ERR_CUDA, "pruner kernel cannot be resident");
    const size_t E0 = ot.size(), I0 = is.size();
    const int span = 8192;
    // Pools: a row that gains entries takes a fresh block, so a pool holds every version of
    // its rows.  At R-MAT scale 20 / 22 the blocks taken add up to about 21 / 29 times the
    // original out-pairs and 22 / 33 times the original in-entries; give each 64 times, within
    // 60% of the free memory.
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
    const size_t wscr_cap = E0 * 16 + (size_t)span * 64;
    const size_t task_cap = (size_t)1 << 22;
    DevBuf db;
    PgParams p;
    std::memset(&p, 0, sizeof(p));
    p.V = V;
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
    if (e == cudaSuccess) e = db.get(&p.rec_off, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.rec_n, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.rt, rec_cap);
    if (e == cudaSuccess) e = db.get(&p.rw, rec_cap);
    if (e == cudaSuccess) e = db.get(&p.rmiss, rec_cap);
    if (e == cudaSuccess) e = db.get(&p.done, (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.resA, 2 * (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.resW, 2 * (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.wmark, 2 * (size_t)V);
    if (e == cudaSuccess) e = db.get(&p.slot_r, (size_t)span * kPgMaxR);
    if (e == cudaSuccess) e = db.get(&p.slot_rn, (size_t)span);
    if (e == cudaSuccess) e = db.get(&p.slot_woff, (size_t)span);
    if (e == cudaSuccess) e = db.get(&p.slot_wn, (size_t)span);
    if (e == cudaSuccess) e = db.get(&p.slot_pass, (size_t)span);
    if (e == cudaSuccess) e = db.get(&p.wscr, wscr_cap);
    if (e == cudaSuccess) e = db.get(&p.task, task_cap);
    if (e == cudaSuccess) e = db.get(&p.ctl, 1);
    C2G_CUDA(e);
    p.out_cap = out_cap;
    p.in_pool_cap = in_cap_pool;
    p.rec_cap = rec_cap;
    p.wscr_cap = wscr_cap;
    p.task_cap = task_cap;
    p.barrier_ns = 20000000000ull;
    p.max_rounds = V + 16;
    // the initial rows
    {
        std::vector<long long> oo((size_t)V), io((size_t)V);
        std::vector<int> on((size_t)V), in_n((size_t)V);
        for (int32_t v = 0; v < V; ++v) {
            oo[v] = orow[v];
            on[v] = orow[v + 1] - orow[v];
            io[v] = irow[v];
            in_n[v] = irow[v + 1] - irow[v];
        }
        const size_t at = I0;
        std::vector<unsigned char> alive(at, 1);
        PgCtl c;
        std::memset(&c, 0, sizeof(c));
        c.out_top = E0;
        c.in_top = (unsigned long long)at;
        c.dmin = V;
        c.round = 1;
        if (E0) {
            C2G_CUDA(cudaMemcpy(p.ot, ot.data(), sizeof(int32_t) * E0, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.ow, ow.data(), sizeof(uint32_t) * E0, cudaMemcpyHostToDevice));
        }
        if (at) {
            C2G_CUDA(cudaMemcpy(p.is, is.data(), sizeof(int32_t) * at, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.ia, alive.data(), at, cudaMemcpyHostToDevice));
        }
        C2G_CUDA(cudaMemcpy(p.out_off, oo.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.out_n, on.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.in_off, io.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.in_n, in_n.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.indeg, in_n.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemset(p.rec_n, 0, sizeof(int) * (size_t)V));
        C2G_CUDA(cudaMemset(p.rec_off, 0, sizeof(long long) * (size_t)V));
        C2G_CUDA(cudaMemset(p.done, 0, (size_t)V));
        C2G_CUDA(cudaMemset(p.resA, 0, sizeof(unsigned long long) * 2 * (size_t)V));
        C2G_CUDA(cudaMemset(p.resW, 0, sizeof(unsigned long long) * 2 * (size_t)V));
        C2G_CUDA(cudaMemset(p.wmark, 0, sizeof(int) * 2 * (size_t)V));
        C2G_CUDA(cudaMemcpy(p.ctl, &c, sizeof(c), cudaMemcpyHostToDevice));
    }
    cudaEvent_t e0, e1;
    C2G_CUDA(cudaEventCreate(&e0));
    C2G_CUDA(cudaEventCreate(&e1));
    void* args[] = {&p};
    cudaEventRecord(e0);
    e = V > 0 ? cudaLaunchCooperativeKernel((const void*)prune_ppr_rounds, dim3(per_sm * sms), dim3(kPgThreads), args, 0,
                                            nullptr)
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
        for (int k = 0; k < 5; ++k) phase_ns[k] = (int64_t)c.phase_ns[k];
    if (c.flags & kPgErrPool) return fail(C2G_ERR_OVERFLOW, "pruner: a row pool ran out");
    if (c.flags & kPgErrRows) return fail(C2G_ERR_FORMAT, "pruner: in-row and out-rows disagree");
    if (c.flags & (C2G_FLAG_BARRIER_TIMEOUT | C2G_FLAG_ITER_CAP) || (V > 0 && !c.finished))
        return fail(C2G_ERR_TIMEOUT, "pruner: rounds did not finish (flags %d)", c.flags);
    // the result, flat: out-rows (vlist, elist, wlist) and the records (hvlist, helist, hwlist)
    std::vector<int> on((size_t)V), rn((size_t)V);
    C2G_CUDA(cudaMemcpy(on.data(), p.out_n, sizeof(int) * (size_t)V, cudaMemcpyDeviceToHost));
    C2G_CUDA(cudaMemcpy(rn.data(), p.rec_n, sizeof(int) * (size_t)V, cudaMemcpyDeviceToHost));
    std::vector<int32_t> pv((size_t)V + 1, 0), hv((size_t)V + 1, 0);
    std::vector<long long> ob((size_t)V), rbase((size_t)V);
    for (int32_t v = 0; v < V; ++v) {
        ob[v] = pv[v];
        rbase[v] = hv[v];
        pv[v + 1] = pv[v] + on[v];
        hv[v + 1] = hv[v] + rn[v];
    }
    const size_t E = (size_t)pv[V], H = (size_t)hv[V];
    DevBuf tmp;
    long long *dob = nullptr, *drb = nullptr;
    int *dpe = nullptr, *dhe = nullptr;
    unsigned *dpw = nullptr, *dhw = nullptr;
    e = tmp.get(&dob, (size_t)V);
    if (e == cudaSuccess) e = tmp.get(&drb, (size_t)V);
    if (e == cudaSuccess) e = tmp.get(&dpe, E);
    if (e == cudaSuccess) e = tmp.get(&dpw, E);
    if (e == cudaSuccess) e = tmp.get(&dhe, H);
    if (e == cudaSuccess) e = tmp.get(&dhw, H);
    C2G_CUDA(e);
    C2G_CUDA(cudaMemcpy(dob, ob.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
    C2G_CUDA(cudaMemcpy(drb, rbase.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
    if (V > 0) {
        pg_gather_rows<<<sms * 8, 256>>>(p.out_off, p.out_n, dob, V, p.ot, p.ow, dpe, dpw);
        pg_gather_rows<<<sms * 8, 256>>>(p.rec_off, p.rec_n, drb, V, p.rt, p.rw, dhe, dhw);
        C2G_CUDA(cudaGetLastError());
    }
    C2G_CUDA(cudaDeviceSynchronize());
    // the files, the device arrays streamed through a pinned staging buffer
    const size_t stage_n = (size_t)1 << 24;
    void* stage = nullptr;
    C2G_CUDA(cudaMallocHost(&stage, 4 * stage_n));
    struct FreeHost {
        void* q;
        ~FreeHost() { cudaFreeHost(q); }
    } free_stage{stage};
    auto put = [&](const std::string& path, const void* dev, size_t n) -> int {
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
    };
    const std::string s = dir + "/ppr/";
    if ((rc = make_dir(dir + "/ppr"))) return rc;
    if ((rc = write_array4(s + "hvlist.bin", hv.data(), hv.size()))) return rc;
    if ((rc = put(s + "helist.bin", dhe, H))) return rc;
    if ((rc = put(s + "hwlist.bin", dhw, H))) return rc;
    if ((rc = write_array4(s + "vlist.bin", pv.data(), pv.size()))) return rc;
    if ((rc = put(s + "elist.bin", dpe, E))) return rc;
    if ((rc = put(s + "wlist.bin", dpw, E))) return rc;
    return C2G_OK;
}

}  // namespace c2g

extern "C" int c2g_prune_ppr_device(const char* dir, double alpha, int device, float* ms, int32_t* rounds,
                                    int64_t* phase_ns) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "prune: dir is NULL");
    if (!(alpha > 0.0 && alpha < 1.0)) return c2g::fail(C2G_ERR_ARG, "prune: alpha must be in (0, 1)");
    return c2g::prune_ppr_device_dir(dir, 1.0 - alpha, device, ms, rounds, phase_ns);
}
