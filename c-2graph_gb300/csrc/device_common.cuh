// Device building blocks shared by the traversal kernels (sm_103a):
//   * a bounded grid barrier for persistent cooperative launches,
//   * L2-coherent loads for data other CTAs write during a launch,
//   * the warp-aggregated frontier append that also writes the edge-tile markers.
//
// The reference synchronises its 20 persistent CTAs with unbounded spins on volatile
// counters (src/sssp/purn/Main.cu:173-189,336-347,379-383) and compacts the frontier
// with a full-V BlockScan sweep every round (src/sssp/purn/Main.cu:350-377).  Here the
// launch is cooperative (co-residency guaranteed), every wait has a time limit after
// which the kernel records C2G_FLAG_BARRIER_TIMEOUT and returns, and the next frontier
// is appended sparsely as vertices improve.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/c2graph.h"

namespace c2g {

constexpr unsigned kFull = 0xffffffffu;
constexpr int kInfDist = 1999999999;  // unreachable distance, src/sssp/base/Main.cu:121

struct GridBarrier {
    unsigned count;
    unsigned gen;
};

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release_u32(unsigned* p, unsigned v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned atom_add_acq_rel_u32(unsigned* p, unsigned v) {
    unsigned old;
    asm volatile("atom.acq_rel.gpu.global.add.u32 %0, [%1], %2;" : "=r"(old) : "l"(p), "r"(v) : "memory");
    return old;
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// L2-coherent loads (bypass L1): for arrays written by other CTAs in the same launch.
__device__ __forceinline__ int ldcg(const int* p) { return __ldcg(p); }
__device__ __forceinline__ unsigned ldcg(const unsigned* p) { return __ldcg(p); }
__device__ __forceinline__ float ldcg(const float* p) { return __ldcg(p); }
__device__ __forceinline__ int2 ldcg(const int2* p) { return __ldcg(p); }
__device__ __forceinline__ unsigned long long ldcg(const unsigned long long* p) { return __ldcg(p); }
__device__ __forceinline__ double ldcg(const double* p) { return __ldcg(p); }
__device__ __forceinline__ float2 ldcg(const float2* p) { return __ldcg(p); }
__device__ __forceinline__ uint4 ldcg(const uint4* p) { return __ldcg(p); }

// Grid barrier with a time limit.  Every CTA of a cooperative launch calls it; it
// returns false (and all later calls return false) once any CTA has given up, so the
// caller returns and the launch ends with C2G_FLAG_BARRIER_TIMEOUT recorded.
// `extra` > 0 makes the barrier wait for that many blocks beyond the grid, so every wait
// runs out (the failure-detection test of c2g_graph_set_watchdog; no block hangs).
__device__ __forceinline__ bool grid_sync(GridBarrier* b, int* flags, unsigned long long limit_ns,
                                          unsigned extra = 0) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        int ok = 1;
        const unsigned g = ld_acquire_u32(&b->gen);
        // Publish the whole CTA's writes (ordered before this thread by bar.sync) at
        // device scope before arriving.
        __threadfence();
        const unsigned arrived = atom_add_acq_rel_u32(&b->count, 1u);
        if (arrived == gridDim.x - 1 + extra) {
            b->count = 0;
            st_release_u32(&b->gen, g + 1);
        } else {
            const unsigned long long t0 = globaltimer_ns();
            unsigned spins = 0;
            while (ld_acquire_u32(&b->gen) == g) {
                if (++spins > 32) __nanosleep(64);
                if ((spins & 255u) == 0) {
                    if (ld_acquire_u32(reinterpret_cast<unsigned*>(flags)) & C2G_FLAG_BARRIER_TIMEOUT) {
                        ok = 0;
                        break;
                    }
                    if (globaltimer_ns() - t0 > limit_ns) {
                        atomicOr(flags, C2G_FLAG_BARRIER_TIMEOUT);
                        ok = 0;
                        break;
                    }
                }
            }
        }
        if (ok && (ld_acquire_u32(reinterpret_cast<unsigned*>(flags)) & C2G_FLAG_BARRIER_TIMEOUT)) ok = 0;
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Phase timing of a persistent launch, read by c2g_graph_last_phases: block 0's
// thread 0 adds the time since the previous mark to phase_ns[phase].  Called right
// after a grid barrier, so each interval is one phase of the whole grid (wait included).
// Phases: 0 initialisation, 1 frontier build / apply / far-pile filter, 2 expansion / push.
__device__ __forceinline__ void phase_mark(unsigned long long* phase_ns, unsigned long long& t, int phase) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        const unsigned long long now = globaltimer_ns();
        phase_ns[phase] += now - t;
        t = now;
    }
}

// Destination of a frontier append.  Entries are (vertex, base) where base is the
// exclusive prefix of the out-degrees of all entries before it, obtained from one
// 64-bit atomic on ctr = (count << 32) | edge_total, so the frontier's edges form one
// contiguous index range [0, T).  mark[t] receives the entry that owns edge t*TILE,
// which lets a warp start expanding any edge tile without a search.
struct FrontierOut {
    int2* q;                  // entries (vertex, base)
    float* val;               // optional per-entry 32-bit value (batched masks)
    double* vald = nullptr;   // optional per-entry FP64 value (pushed residual)
    int* mark;                // tile -> owning entry
    unsigned long long* ctr;  // packed counter
    unsigned cap;             // entry capacity
    unsigned mark_cap;        // marker capacity
    int log_tile;             // log2(edges per tile)
    int* flags;
};

// Warp-collective count-only append of vertex ids.
__device__ __forceinline__ void list_push(int* list, unsigned* ctr, unsigned cap, int* flags, bool want, int v) {
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(kFull, want);
    if (m == 0) return;
    const int leader = __ffs(m) - 1;
    unsigned old = 0;
    if (lane == leader) old = atomicAdd(ctr, (unsigned)__popc(m));
    old = __shfl_sync(kFull, old, leader);
    if (want) {
        const unsigned slot = old + (unsigned)__popc(m & ((1u << lane) - 1u));
        if (slot < cap)
            list[slot] = v;
        else
            atomicOr(flags, C2G_FLAG_QUEUE_OVERFLOW);
    }
}

// Owner lookup inside a batch of 32 frontier entries held one per lane: the largest
// lane k with base_k <= e (bases strictly increase across valid lanes; invalid lanes
// hold INT_MAX).
__device__ __forceinline__ int owner_lane(unsigned base, unsigned e) {
    int k = 0;
#pragma unroll
    for (int s = 16; s >= 1; s >>= 1) {
        const unsigned b = (unsigned)__shfl_sync(kFull, (int)base, k + s);
        if (b <= e) k += s;
    }
    return k;
}

// Per-warp staging of appends in shared memory.  A warp collects appended entries in a
// 128-entry stage (warp-aggregated with ballot/popc, no atomics) and writes them to the
// global queue with ONE global atomic per flush.  A single global counter hit by every
// warp on every push serialises at its L2 slice; staging cuts those atomics by up to
// 128x.  The stage count n is warp-uniform.
constexpr int kStageCap = 128;

struct WarpStage {
    int* v;    // shared [kStageCap] vertex
    int* d;    // shared [kStageCap] out-degree (frontier stages only)
    float* x;  // shared [kStageCap] value, or nullptr
    int n;
    double* xd = nullptr;  // shared [kStageCap] FP64 value, or nullptr
};

// Write the stage to `out`: entries keep their stage order, so slots and edge bases
// stay monotone, which the owner search of the next round relies on.
__device__ __forceinline__ void stage_flush(WarpStage& st, const FrontierOut& out) {
    const int n = st.n;
    if (n == 0) return;
    __syncwarp();
    const int lane = threadIdx.x & 31;
    int dv[4], dsum = 0;
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = 4 * lane + k;
        dv[k] = i < n ? st.d[i] : 0;
        dsum += dv[k];
    }
    int incl = dsum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int t = __shfl_up_sync(kFull, incl, o);
        if (lane >= o) incl += t;
    }
    const unsigned total = (unsigned)__shfl_sync(kFull, incl, 31);
    unsigned long long old = 0;
    if (lane == 0) old = atomicAdd(out.ctr, ((unsigned long long)n << 32) | (unsigned long long)total);
    old = __shfl_sync(kFull, old, 0);
    const unsigned slot0 = (unsigned)(old >> 32);
    unsigned base = (unsigned)old + (unsigned)(incl - dsum);
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        const int i = 4 * lane + k;
        if (i < n) {
            const unsigned slot = slot0 + (unsigned)i;
            if (slot < out.cap) {
                out.q[slot] = make_int2(st.v[i], (int)base);
                if (out.val) out.val[slot] = st.x[i];
                if (out.vald) out.vald[slot] = st.xd[i];
                const unsigned tile = 1u << out.log_tile;
                const unsigned t0 = (base + tile - 1) >> out.log_tile;
                const unsigned t1 = (base + (unsigned)dv[k] - 1) >> out.log_tile;
                for (unsigned t = t0; t <= t1 && t < out.mark_cap; ++t) out.mark[t] = (int)slot;
            } else {
                atomicOr(out.flags, C2G_FLAG_QUEUE_OVERFLOW);
            }
            base += (unsigned)dv[k];
        }
    }
    st.n = 0;
    __syncwarp();
}

// Warp-collective: lanes with `want` stage (v, deg, x); deg must be > 0.
__device__ __forceinline__ void stage_push(WarpStage& st, const FrontierOut& out, bool want, int v, int deg,
                                           float x, double xd = 0.0) {
    const unsigned m = __ballot_sync(kFull, want);
    if (m == 0) return;
    const int cnt = __popc(m);
    if (st.n + cnt > kStageCap) stage_flush(st, out);
    const int lane = threadIdx.x & 31;
    if (want) {
        const int i = st.n + __popc(m & ((1u << lane) - 1u));
        st.v[i] = v;
        st.d[i] = deg;
        if (st.x) st.x[i] = x;
        if (st.xd) st.xd[i] = xd;
    }
    st.n += cnt;
}

// Stage of a plain id list (count-only counter).
__device__ __forceinline__ void list_stage_flush(WarpStage& st, int* list, unsigned* ctr, unsigned cap, int* flags) {
    const int n = st.n;
    if (n == 0) return;
    __syncwarp();
    const int lane = threadIdx.x & 31;
    unsigned old = 0;
    if (lane == 0) old = atomicAdd(ctr, (unsigned)n);
    old = __shfl_sync(kFull, old, 0);
    for (int i = lane; i < n; i += 32) {
        if (old + (unsigned)i < cap)
            list[old + (unsigned)i] = st.v[i];
        else
            atomicOr(flags, C2G_FLAG_QUEUE_OVERFLOW);
    }
    st.n = 0;
    __syncwarp();
}

__device__ __forceinline__ void list_stage_push(WarpStage& st, int* list, unsigned* ctr, unsigned cap, int* flags,
                                                bool want, int v) {
    const unsigned m = __ballot_sync(kFull, want);
    if (m == 0) return;
    const int cnt = __popc(m);
    if (st.n + cnt > kStageCap) list_stage_flush(st, list, ctr, cap, flags);
    const int lane = threadIdx.x & 31;
    if (want) st.v[st.n + __popc(m & ((1u << lane) - 1u))] = v;
    st.n += cnt;
}

// Shared-memory backing for two stages per warp (512-thread blocks: 16 warps).
struct StageSmem {
    int v0[16][kStageCap];
    int d0[16][kStageCap];
    float x0[16][kStageCap];
    int v1[16][kStageCap];
};

// Stage backing for the push kernels: FP64 values instead of 32-bit ones.
struct StageSmemD {
    int v0[16][kStageCap];
    int d0[16][kStageCap];
    double xd0[16][kStageCap];
    int v1[16][kStageCap];
};

// Next tile of a round for this warp from the round's tile counter (lane 0 takes it, the
// warp shares it).  Where tiles differ in cost, or are few, a dynamic queue balances the
// warps better than a fixed round-robin.
__device__ __forceinline__ unsigned next_tile(unsigned* ctr, int lane) {
    unsigned t = 0;
    if (lane == 0) t = atomicAdd(ctr, 1u);
    return (unsigned)__shfl_sync(kFull, (int)t, 0);
}

// Warp-cooperative walk over the edges of a frontier, in tiles of 2^log_tile edges
// assigned to warps round-robin (tile t goes to warp t mod nwarps, no shared counter).
// For each group of 32*U edges every lane gets U edges (stride 32, so the warp reads
// consecutive (target, weight) pairs) and calls
//     body(ok[U], idx[U], val[U])   (val: the owner value type, int or double)
// where idx is the edge's index in the adjacency array, ok says whether the lane holds
// an edge, and val is owner_val(vertex, entry) of the edge's owning frontier entry.
// body must be warp-collective-safe: every lane of the warp calls it.
template <int U, typename OwnerVal, typename Body>
__device__ __forceinline__ void walk_frontier_edges(const int2* __restrict__ q, const int* __restrict__ mark,
                                                    const int* __restrict__ row, unsigned F, unsigned T,
                                                    int log_tile, unsigned mark_cap, unsigned qcap, unsigned E,
                                                    int* flags, OwnerVal owner_val, Body body,
                                                    unsigned* tctr = nullptr) {
    using VT = decltype(owner_val(0, 0u));  // int or double
    const int lane = threadIdx.x & 31;
    const unsigned gwarp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned tw = 1u << log_tile;
    const unsigned ntiles = (T + tw - 1) >> log_tile;
    if (ntiles > mark_cap || F > qcap || T > E) {
        if (lane == 0) atomicOr(flags, C2G_FLAG_BOUNDS);
        return;
    }
    // tctr: a round's tile counter (zero at the round's start) for a dynamic queue of
    // tiles, the next one fetched while the current one runs; nullptr: round-robin.
    unsigned tn = tctr ? next_tile(tctr, lane) : gwarp;
    for (unsigned t = tn; t < ntiles; t = tn) {
        tn = tctr ? next_tile(tctr, lane) : t + nwarps;
        unsigned e0 = t << log_tile;
        const unsigned e1 = min(e0 + tw, T);
        unsigned o = (unsigned)ldcg(mark + t);
        while (e0 < e1) {
            // One frontier entry per lane: its edge range [base, end) and owner value.
            const unsigned j = o + (unsigned)lane;
            unsigned base = 0x7fffffffu, endv = 0xffffffffu;
            int rs = 0;
            VT val = VT(0);
            if (j < F) {
                const int2 qe = ldcg(q + j);
                base = (unsigned)qe.y;
                rs = __ldg(row + qe.x);
                endv = base + (unsigned)(__ldg(row + qe.x + 1) - rs);
                val = owner_val(qe.x, j);
            }
            const unsigned seg_end = min(e1, (unsigned)__shfl_sync(kFull, endv, 31));
            if (seg_end <= e0 || o >= F) {  // the tile marker did not lead to its owner
                if (lane == 0) atomicOr(flags, C2G_FLAG_BOUNDS);
                break;
            }
            for (unsigned eb = e0; eb < seg_end; eb += 32u * U) {
                bool ok[U];
                unsigned idx[U];
                VT sv[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const unsigned e = eb + (unsigned)lane + 32u * u;
                    const int k = owner_lane(base, e);
                    const unsigned srs = (unsigned)__shfl_sync(kFull, rs, k);
                    const unsigned sb = (unsigned)__shfl_sync(kFull, (int)base, k);
                    sv[u] = __shfl_sync(kFull, val, k);
                    idx[u] = srs + (e - sb);
                    ok[u] = e < seg_end && sb <= e && idx[u] < E;
                    if (e < seg_end && !ok[u]) atomicOr(flags, C2G_FLAG_BOUNDS);
                }
                body(ok, idx, sv);
            }
            e0 = seg_end;
            o += 32;
        }
    }
}

}  // namespace c2g
