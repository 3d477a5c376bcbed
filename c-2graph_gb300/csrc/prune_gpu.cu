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
// a window plans its visit on the current state (the rows it reads and would write) and
// reserves those rows under its id; it commits when no earlier candidate of the window
// writes a row it reads or touches a row it writes, unless an earlier candidate that
// failed had a row it reads written in this round (its plan may change), past which
// nothing commits.  The first unvisited vertex always commits, so every round makes
// progress.  Committed visits touch disjoint rows and run in parallel, one warp each, with
// the reference's steps: roots in in-row order, membership of each out-edge's target in
// every root's sorted row, the in-row updates of the moved targets in out-row order (lane
// 0: a moved pair can repeat a target), and a sorted merge of the moved pairs into each
// root's row with the weight (w * keep) * w' in double, rounded to float.  Rows live in
// device pools; a merge or a grown in-row takes a new block from the pool (bump
// allocation), so no row is ever shared.  The schedule is the one orc_prune_ppr_speculative
// checks on the CPU.
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
                           std::vector<uint32_t>& ow, std::vector<int32_t>& irow, std::vector<int32_t>& is);

constexpr int kPgThreads = 256;
constexpr int kPgMaxRoots = 5;  // the in-degree bound of purn-ppr (src/purn-ppr.cpp:146-152)
constexpr int kPgMaxR = 2 + kPgMaxRoots;  // rows a visit reads: its in-row, its out-row, its roots' out-rows

struct PgCtl {
    unsigned bar_count, bar_gen;  // GridBarrier
    int flags;
    int pos;    // the first unvisited vertex
    int dmin;   // this round: the first failed candidate whose reads a committer writes
    int round;
    int finished;
    int pad;
    unsigned long long out_top, in_top, rec_top, wscr_top;  // pool bump pointers
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
    int* in_cap;
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
    long long* slot_woff;      // rows written, in wscr
    int* slot_wn;
    unsigned char* slot_pass;
    int* wscr;
    unsigned long long wscr_cap;
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

// first index of row [off, off + n) of `t` with t >= key, or n
__device__ __forceinline__ int pg_lower(const int* t, long long off, int n, int key) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (ldcg(t + off + mid) < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

// The live roots of i in in-row order (every lane gets them).  Returns their count.
__device__ int pg_roots(const PgParams& p, int i, int* rt, int lane) {
    const long long off = ldl(p.in_off + i);
    const int n = ldcg(p.in_n + i);
    int nr = 0;
    for (int b = 0; b < n && nr <= kPgMaxRoots; b += 32) {
        const int k = b + lane;
        const bool a = k < n && ldb(p.ia + off + k) != 0;
        const int s = k < n ? ldcg(p.is + off + k) : 0;
        unsigned m = __ballot_sync(kFull, a);
        while (m && nr <= kPgMaxRoots) {
            const int src = __shfl_sync(kFull, s, __ffs(m) - 1);
            if (nr < kPgMaxRoots) rt[nr] = src;
            ++nr;
            m &= m - 1u;
        }
    }
    return nr;
}

__device__ __forceinline__ bool pg_member(const PgParams& p, int r, int v) {
    const long long off = ldl(p.out_off + r);
    const int n = ldcg(p.out_n + r);
    const int k = pg_lower(p.ot, off, n, v);
    return k < n && ldcg(p.ot + off + k) == v;
}

// Does the edge i -> v move (every root but at most one has v)?  miss: roots without v.
__device__ __forceinline__ bool pg_moves(const PgParams& p, const int* rt, int j, int v, unsigned& miss) {
    miss = 0u;
    for (int k = 0; k < j; ++k)
        if (rt[k] == v) return false;  // a root keeps its edge
    int cnt = 0;
    for (int k = 0; k < j; ++k) {
        if (pg_member(p, rt[k], v))
            ++cnt;
        else
            miss |= 1u << k;
    }
    return cnt + 2 > j;
}

__device__ __forceinline__ bool pg_prunes(const PgParams& p, int i) {
    const int d = ldcg(p.indeg + i);
    return ldcg(p.out_n + i) > 0 && d > 0 && d <= kPgMaxRoots;
}

// Plan of candidate i (slot c): the rows it reads and the rows it would write; reserve them.
__device__ void pg_plan(const PgParams& p, int i, int c, int round, int lane) {
    const int V = p.V;
    int* R = p.slot_r + (size_t)c * kPgMaxR;
    int rn = 2;
    if (lane == 0) {
        R[0] = V + i;
        R[1] = i;
    }
    long long woff = 0;
    int wn = 0;
    if (pg_prunes(p, i)) {
        int rt[kPgMaxRoots];
        const int nr = pg_roots(p, i, rt, lane);
        const int j = min(nr, kPgMaxRoots);
        if (lane == 0)
            for (int k = 0; k < j; ++k) R[2 + k] = rt[k];
        rn = 2 + j;
        const long long off = ldl(p.out_off + i);
        const int on = ldcg(p.out_n + i);
        unsigned long long wb = 0;
        if (lane == 0) wb = atomicAdd(&p.ctl->wscr_top, (unsigned long long)on + 8ull);
        wb = __shfl_sync(kFull, wb, 0);
        if (wb + (unsigned long long)on + 8ull > p.wscr_cap) {
            if (lane == 0) atomicOr(&p.ctl->flags, kPgErrPool);
            wn = 0;
        } else {
            woff = (long long)wb;
            for (int b = 0; b < on; b += 32) {
                const int e = b + lane;
                unsigned miss;
                const bool mv = e < on && pg_moves(p, rt, j, ldcg(p.ot + off + e), miss);
                const unsigned m = __ballot_sync(kFull, mv);
                if (mv) p.wscr[woff + wn + __popc(m & ((1u << lane) - 1u))] = V + ldcg(p.ot + off + e);
                wn += __popc(m);
            }
            if (wn > 0) {  // it moves edges: its out-row and its roots' out-rows change
                if (lane == 0) {
                    p.wscr[woff + wn] = i;
                    for (int k = 0; k < j; ++k) p.wscr[woff + wn + 1 + k] = rt[k];
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
    if (lane < rn) atomicMax(p.resA + R[lane], key);
    for (int k = lane; k < wn; k += 32) {
        const int r = p.wscr[woff + k];
        atomicMax(p.resA + r, key);
        atomicMax(p.resW + r, key);
    }
}

// A committed visit of vertex i (the reference's steps; the plan's rows are unchanged).
__device__ void pg_visit(const PgParams& p, int i, int lane) {
    int rt[kPgMaxRoots];
    const int nr = pg_roots(p, i, rt, lane);
    const int j = ldcg(p.indeg + i);
    if (nr != j || j > kPgMaxRoots) {  // the reference stops on this (something error2)
        if (lane == 0) atomicOr(&p.ctl->flags, kPgErrRows);
        return;
    }
    // dis[k]: weight of root k -> i, its first pair with target i
    unsigned dis[kPgMaxRoots];
    for (int k = 0; k < j; ++k) {
        unsigned d = 0u;
        if (lane == 0) {
            const long long off = ldl(p.out_off + rt[k]);
            const int n = ldcg(p.out_n + rt[k]);
            const int q = pg_lower(p.ot, off, n, i);
            if (q < n && ldcg(p.ot + off + q) == i)
                d = ldcg(p.ow + off + q);
            else
                atomicOr(&p.ctl->flags, kPgErrRows);
        }
        dis[k] = (unsigned)__shfl_sync(kFull, (int)d, 0);
    }
    const long long ooff = ldl(p.out_off + i);
    const int on = ldcg(p.out_n + i);
    unsigned long long rb = 0;
    if (lane == 0) rb = atomicAdd(&p.ctl->rec_top, (unsigned long long)on);
    rb = __shfl_sync(kFull, rb, 0);
    if (rb + (unsigned long long)on > p.rec_cap) {
        if (lane == 0) atomicOr(&p.ctl->flags, kPgErrPool);
        return;
    }
    // split the out-row: moved pairs to the record (in order), kept ones compacted in place
    int nrm = 0, kn = 0;
    for (int b = 0; b < on; b += 32) {
        const int e = b + lane;
        const bool valid = e < on;
        const int v = valid ? ldcg(p.ot + ooff + e) : 0;
        const unsigned d3 = valid ? ldcg(p.ow + ooff + e) : 0u;
        unsigned miss = 0u;
        const bool mv = valid && pg_moves(p, rt, j, v, miss);
        const bool kp = valid && !mv;
        const unsigned mm = __ballot_sync(kFull, mv), mk = __ballot_sync(kFull, kp);
        const unsigned lt = (1u << lane) - 1u;
        if (mv) {
            const long long at = (long long)rb + nrm + __popc(mm & lt);
            p.rt[at] = v;
            p.rw[at] = d3;
            p.rmiss[at] = (unsigned char)miss;
        }
        __syncwarp();  // every lane has read its pair before the compaction writes
        if (kp) {
            const long long at = ooff + kn + __popc(mk & lt);
            p.ot[at] = v;
            p.ow[at] = d3;
        }
        nrm += __popc(mm);
        kn += __popc(mk);
        __syncwarp();
    }
    // in-rows of the moved targets, in out-row order: every root without the target gains
    // it (a new entry or a revived one), and i dies in it (src/purn-ppr.cpp:196-236)
    if (lane == 0) {
        for (int k = 0; k < nrm; ++k) {
            const int v = ldcg(p.rt + rb + k);
            const unsigned miss = ldb(p.rmiss + rb + k);
            for (int q = 0; q < j; ++q) {
                if (!((miss >> q) & 1u)) continue;
                const int r = rt[q];
                long long off = ldl(p.in_off + v);
                int n = ldcg(p.in_n + v);
                const int at = pg_lower(p.is, off, n, r);
                if (at < n && ldcg(p.is + off + at) == r) {
                    if (!ldb(p.ia + off + at)) {
                        p.ia[off + at] = 1;
                        p.indeg[v] = ldcg(p.indeg + v) + 1;
                    }
                    continue;
                }
                if (n < ldcg(p.in_cap + v)) {  // room in place: shift the tail
                    for (int x = n; x > at; --x) {
                        p.is[off + x] = ldcg(p.is + off + x - 1);
                        p.ia[off + x] = ldb(p.ia + off + x - 1);
                    }
                } else {  // a new block twice the size
                    const int cap = 2 * n + 4;
                    const unsigned long long nb = atomicAdd(&p.ctl->in_top, (unsigned long long)cap);
                    if (nb + (unsigned long long)cap > p.in_pool_cap) {
                        atomicOr(&p.ctl->flags, kPgErrPool);
                        return;
                    }
                    const long long noff = (long long)nb;
                    for (int x = 0; x < at; ++x) {
                        p.is[noff + x] = ldcg(p.is + off + x);
                        p.ia[noff + x] = ldb(p.ia + off + x);
                    }
                    for (int x = at; x < n; ++x) {
                        p.is[noff + x + 1] = ldcg(p.is + off + x);
                        p.ia[noff + x + 1] = ldb(p.ia + off + x);
                    }
                    off = noff;
                    p.in_off[v] = noff;
                    p.in_cap[v] = cap;
                }
                p.is[off + at] = r;
                p.ia[off + at] = 1;
                p.in_n[v] = n + 1;
                p.indeg[v] = ldcg(p.indeg + v) + 1;
            }
            const long long off = ldl(p.in_off + v);
            const int n = ldcg(p.in_n + v);
            const int at = pg_lower(p.is, off, n, i);
            if (at >= n || ldcg(p.is + off + at) != i) {
                atomicOr(&p.ctl->flags, kPgErrRows);
                return;
            }
            p.indeg[v] = ldcg(p.indeg + v) - 1;
            p.ia[off + at] = 0;
        }
    }
    // the moved pairs merge into every root's sorted row, one lane per root
    if (nrm > 0 && lane < j) {
        const int r = rt[lane];
        const double dk = (double)__uint_as_float(dis[lane]);
        const long long off = ldl(p.out_off + r);
        const int n = ldcg(p.out_n + r);
        const unsigned long long nb = atomicAdd(&p.ctl->out_top, (unsigned long long)(n + nrm));
        if (nb + (unsigned long long)(n + nrm) > p.out_cap) {
            atomicOr(&p.ctl->flags, kPgErrPool);
        } else {
            const long long noff = (long long)nb;
            int a = 0, b = 0, m = 0;
            while (a < n || b < nrm) {
                const int ta = a < n ? ldcg(p.ot + off + a) : 0;
                const int tb = b < nrm ? ldcg(p.rt + rb + b) : 0;
                if (a < n && (b == nrm || ta < tb)) {
                    p.ot[noff + m] = ta;
                    p.ow[noff + m] = ldcg(p.ow + off + a);
                    ++a;
                } else if (a < n && ta == tb) {  // (double)old + (w * keep) * w', to float
                    const double f = __dmul_rn(__dmul_rn((double)__uint_as_float(ldcg(p.rw + rb + b)), p.keep), dk);
                    p.ot[noff + m] = ta;
                    p.ow[noff + m] =
                        __float_as_uint(__double2float_rn(__dadd_rn((double)__uint_as_float(ldcg(p.ow + off + a)), f)));
                    ++a;
                    ++b;
                } else {  // a new pair: (w * keep) * w', to float
                    const double f = __dmul_rn(__dmul_rn((double)__uint_as_float(ldcg(p.rw + rb + b)), p.keep), dk);
                    p.ot[noff + m] = tb;
                    p.ow[noff + m] = __float_as_uint(__double2float_rn(f));
                    ++b;
                }
                ++m;
            }
            p.out_off[r] = noff;
            p.out_n[r] = m;
        }
    }
    if (lane == 0) {
        p.out_n[i] = kn;
        p.rec_off[i] = (long long)rb;
        p.rec_n[i] = nrm;
    }
}

__global__ void __launch_bounds__(kPgThreads) prune_ppr_rounds(const PgParams p) {
    PgCtl* ctl = p.ctl;
    GridBarrier* bar = reinterpret_cast<GridBarrier*>(&ctl->bar_count);
    int* flags = &ctl->flags;
    const int lane = threadIdx.x & 31;
    const unsigned gtid = blockIdx.x * blockDim.x + threadIdx.x;
    const int gwarp = (int)(gtid >> 5), nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int guard = 0; guard < p.max_rounds; ++guard) {
        const int pos = ldcg(&ctl->pos), round = ldcg(&ctl->round);
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
        // commit
        const int dmin = ldcg(&ctl->dmin);
        for (int c = gwarp; c < p.span; c += nwarps) {
            const int i = pos + c;
            if (i >= p.V || i > dmin) break;
            if (ldcg(p.slot_rn + c) < 0 || !ldb(p.slot_pass + c)) continue;
            if (pg_prunes(p, i)) pg_visit(p, i, lane);
            if (lane == 0) p.done[i] = 1;
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
        // next window
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
                if (q >= p.V) ctl->finished = 1;
            }
        }
        if (!grid_sync(bar, flags, p.barrier_ns)) return;
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

static int prune_ppr_device_dir(const std::string& dir, double keep, int device, float* ms, int* rounds) {
    int32_t V = 0;
    std::vector<int32_t> orow, ot, irow, is;
    std::vector<uint32_t> ow;
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
    // pools: the rows a merge or an in-row growth writes anew take fresh blocks
    size_t free_b = 0, total_b = 0;
    C2G_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const size_t want_out = E0 * 48 + (1u << 20);
    const size_t out_cap = std::min(want_out, (size_t)(0.45 * (double)free_b) / 8);
    const size_t in_cap_pool = I0 * 8 + (1u << 20);
    const size_t rec_cap = E0 * 6 + (1u << 20);
    const size_t wscr_cap = E0 * 2 + (size_t)span * 16;
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
    if (e == cudaSuccess) e = db.get(&p.in_cap, (size_t)V);
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
    if (e == cudaSuccess) e = db.get(&p.ctl, 1);
    C2G_CUDA(e);
    p.out_cap = out_cap;
    p.in_pool_cap = in_cap_pool;
    p.rec_cap = rec_cap;
    p.wscr_cap = wscr_cap;
    p.barrier_ns = 20000000000ull;
    p.max_rounds = V + 16;
    // the initial rows: in-rows get room for two insertions each before they move
    {
        std::vector<long long> oo((size_t)V), io((size_t)V);
        std::vector<int> on((size_t)V), in_n((size_t)V), ic((size_t)V), deg((size_t)V);
        std::vector<int32_t> is2(in_cap_pool < I0 + 2 * (size_t)V ? 0 : I0 + 2 * (size_t)V);
        if (is2.empty()) return fail(C2G_ERR_RANGE, "pruner: in-row pool too small");
        long long at = 0;
        for (int32_t v = 0; v < V; ++v) {
            oo[v] = orow[v];
            on[v] = orow[v + 1] - orow[v];
            in_n[v] = irow[v + 1] - irow[v];
            deg[v] = in_n[v];
            io[v] = at;
            ic[v] = in_n[v] + 2;
            std::copy(is.begin() + irow[v], is.begin() + irow[v + 1], is2.begin() + at);
            at += ic[v];
        }
        std::vector<unsigned char> alive((size_t)at, 1);
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
            C2G_CUDA(cudaMemcpy(p.is, is2.data(), sizeof(int32_t) * (size_t)at, cudaMemcpyHostToDevice));
            C2G_CUDA(cudaMemcpy(p.ia, alive.data(), (size_t)at, cudaMemcpyHostToDevice));
        }
        C2G_CUDA(cudaMemcpy(p.out_off, oo.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.out_n, on.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.in_off, io.data(), sizeof(long long) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.in_n, in_n.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.in_cap, ic.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
        C2G_CUDA(cudaMemcpy(p.indeg, deg.data(), sizeof(int) * (size_t)V, cudaMemcpyHostToDevice));
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
    std::vector<int32_t> pe(E), he(H);
    std::vector<uint32_t> pw(E), hw(H);
    {
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
        if (E) {
            C2G_CUDA(cudaMemcpy(pe.data(), dpe, sizeof(int32_t) * E, cudaMemcpyDeviceToHost));
            C2G_CUDA(cudaMemcpy(pw.data(), dpw, sizeof(uint32_t) * E, cudaMemcpyDeviceToHost));
        }
        if (H) {
            C2G_CUDA(cudaMemcpy(he.data(), dhe, sizeof(int32_t) * H, cudaMemcpyDeviceToHost));
            C2G_CUDA(cudaMemcpy(hw.data(), dhw, sizeof(uint32_t) * H, cudaMemcpyDeviceToHost));
        }
    }
    const std::string s = dir + "/ppr/";
    if ((rc = make_dir(dir + "/ppr"))) return rc;
    if ((rc = write_array4(s + "hvlist.bin", hv.data(), hv.size()))) return rc;
    if ((rc = write_array4(s + "helist.bin", he.data(), he.size()))) return rc;
    if ((rc = write_array4(s + "hwlist.bin", hw.data(), hw.size()))) return rc;
    if ((rc = write_array4(s + "vlist.bin", pv.data(), pv.size()))) return rc;
    if ((rc = write_array4(s + "elist.bin", pe.data(), pe.size()))) return rc;
    if ((rc = write_array4(s + "wlist.bin", pw.data(), pw.size()))) return rc;
    return C2G_OK;
}

}  // namespace c2g

extern "C" int c2g_prune_ppr_device(const char* dir, double alpha, int device, float* ms, int32_t* rounds) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "prune: dir is NULL");
    if (!(alpha > 0.0 && alpha < 1.0)) return c2g::fail(C2G_ERR_ARG, "prune: alpha must be in (0, 1)");
    return c2g::prune_ppr_device_dir(dir, 1.0 - alpha, device, ms, rounds);
}
