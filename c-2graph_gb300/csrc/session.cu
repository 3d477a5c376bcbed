// Resident batches ("sessions"): slot-level continuous batching with device-resident
// snapshot / evict of per-query state.
//
// The reference's C^2graph-PM mode runs a query for a few GPU iterations, then ships its
// distances (or residuals) and frontier through a pinned ring of `Data` slots to a CPU
// thread that finishes it (src/sssp/purn-perk/SSSP.h:13-29, src/sssp/purn-perk/Main.cu:
// 87-246).  Here a session keeps Q query slots of the batched kernels resident on the
// device and runs them in epochs of a bounded number of rounds:
//   * between epochs the whole state rests in the [V][Q] arrays (SSSP: distances and the
//     next round's improvement masks; PPR: pr, res, the pushed residuals and activity
//     masks of the frontier, the dangling-lane masks), so each epoch starts where the
//     previous one stopped and every query follows exactly its own rounds;
//   * a query admitted while others run takes a free slot and joins at the next epoch
//     (its column is reset and its source activated); a query whose lanes are no longer
//     active after an epoch is finished and its slot is freed when its result is read;
//   * a running query can be evicted: its column and its frontier lanes are copied into a
//     device-resident snapshot and its lanes leave the frontier; resuming the snapshot in
//     any free slot (of this or another session on the same graph) continues the same
//     rounds.
// SSSP distances do not depend on the schedule (the int32 fixed point is unique); a PPR
// query runs the same BSP rounds as c2g_ppr / c2g_ppr_batch in base mode (FP32 result
// within summation order).  PPR round caps are per query: an epoch never runs a query past
// its cap, and a query reaching it keeps its frontier residuals, as c2g_ppr_batch does.
#include <climits>
#include <cstring>
#include <mutex>
#include <vector>

#include "device_common.cuh"
#include "fp64_mul.h"
#include "internal.h"

namespace c2g {
int graph_view(c2g_graph* base, c2g_graph** out);
void graph_free_view(c2g_graph* g);
}  // namespace c2g

using namespace c2g;

namespace {

// ---- kernels ------------------------------------------------------------------------------

// Reset the columns of joining slots: SSSP distances to unreachable, PPR pr / res to 0.
__global__ void join_cols_kernel(int* dist, float* pr, double* res, int Q, long long V, const int2* joins, int n) {
    const long long total = V * (long long)n;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const long long v = i / n;
        const int slot = joins[i - v * n].x;
        const size_t off = (size_t)v * (size_t)Q + (size_t)slot;
        if (dist) dist[off] = kInfDist;
        if (pr) pr[off] = 0.f;
        if (res) res[off] = 0.0;
    }
}

// Sources of joining SSSP slots: distance 0, marked for the next sweep.
__global__ void sssp_join_src_kernel(int* dist, unsigned* mask, int Q, int logW, const int2* joins, int n) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int slot = joins[i].x, s = joins[i].y;
    dist[(size_t)s * (size_t)Q + (size_t)slot] = 0;
    atomicOr(mask + ((size_t)s << logW) + (slot >> 5), 1u << (slot & 31));
}

__device__ __forceinline__ float2 rq_pair(double q) {
    if (c2g_split_ok(q)) {
        const c2g_pair hl = c2g_split_pair(q);
        return make_float2(c2g_bitsf(hl.hi), c2g_bitsf(hl.lo));
    }
    const float hi = __double2float_rz(q);
    return make_float2(hi, __double2float_rz(q - (double)hi));
}

// Sources of joining PPR slots (base mode, src/ppr/base/Main.cu:146-150): pr = pr0 and the
// source activated with residual r0, as the first sweep of c2g_ppr_batch activates it: a
// source with out-edges pushes (1 - alpha) r0 next round, one without keeps r0 until it is
// popped.
__global__ void ppr_join_src_kernel(PprBatchArrays a, int b, int Q, int logW, const int* row, const int2* joins, int n,
                                    float alpha, float r0, float pr0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int slot = joins[i].x, s = joins[i].y;
    const size_t off = (size_t)s * (size_t)Q + (size_t)slot;
    const size_t wi = ((size_t)s << logW) + (size_t)(slot >> 5);
    const unsigned bit = 1u << (slot & 31);
    a.pr[off] = pr0;
    if (row[s + 1] - row[s] > 0) {
        const double q = (1.0 - (double)alpha) * (double)r0;
        a.rq[b][off] = q;
        a.rqf[b][off] = rq_pair(q);
        a.res[off] = 0.0;
        atomicOr(a.amask[b] + wi, bit);
    } else {
        a.res[off] = (double)r0;
        atomicOr(a.dmask + wi, bit);
    }
}

// Lanes with any bit in the masks (per query word): OR over all vertices.  Every thread
// sees one word index (the stride is a multiple of W <= 32).
__global__ void active_scan_kernel(const unsigned* m0, const unsigned* m1, size_t n, int W, unsigned* out) {
    unsigned acc = 0u;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        acc |= __ldg(m0 + i);
        if (m1) acc |= __ldg(m1 + i);
    }
    for (int o = 16; o >= W; o >>= 1) acc |= __shfl_xor_sync(kFull, acc, o);
    const int lane = threadIdx.x & 31;
    if (lane < W && acc) atomicOr(out + lane, acc);
}

// One column of a [V][Q] array into a dense vector (device or mapped host memory).
template <typename S, typename D>
__global__ void gather_col_kernel(const S* src, int Q, int V, int slot, D* out) {
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride)
        out[v] = (D)src[(size_t)v * (size_t)Q + (size_t)slot];
}

// Snapshot of a slot's lanes in a [V][W] mask array as a V-bit map (bit v of word v/32);
// with `clear` the lanes leave the mask.  One warp per 32 vertices.
__device__ __forceinline__ void snap_bits(unsigned* mask, int logW, int V, int slot, bool clear, unsigned* bits) {
    const int lane = threadIdx.x & 31;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned bit = 1u << (slot & 31);
    for (int b = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; b * 32 < V; b += nwarps) {
        const int v = b * 32 + lane;
        bool on = false;
        if (v < V) {
            unsigned* m = mask + ((size_t)v << logW) + (size_t)(slot >> 5);
            on = (__ldcg(m) & bit) != 0u;
            if (on && clear) atomicAnd(m, ~bit);
        }
        const unsigned word = __ballot_sync(kFull, on);
        if (lane == 0) bits[b] = word;
    }
}

__global__ void snap_bits_kernel(unsigned* mask, int logW, int V, int slot, int clear, unsigned* bits) {
    snap_bits(mask, logW, V, slot, clear != 0, bits);
}

// Restore a slot's lanes from a V-bit map.
__global__ void restore_bits_kernel(unsigned* mask, int logW, int V, int slot, const unsigned* bits) {
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride)
        if ((bits[v >> 5] >> (v & 31)) & 1u) atomicOr(mask + ((size_t)v << logW) + (size_t)(slot >> 5), 1u << (slot & 31));
}

// Copy a dense vector into a column (and, for pushed residuals, their float pairs).
template <typename T>
__global__ void scatter_col_kernel(T* dst, int Q, int V, int slot, const T* col) {
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride)
        dst[(size_t)v * (size_t)Q + (size_t)slot] = col[v];
}

__global__ void scatter_rq_kernel(double* rq, float2* rqf, int Q, int V, int slot, const double* col,
                                  const unsigned* bits) {
    const int stride = gridDim.x * blockDim.x;
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride)
        if ((bits[v >> 5] >> (v & 31)) & 1u) {
            const size_t off = (size_t)v * (size_t)Q + (size_t)slot;
            rq[off] = col[v];
            rqf[off] = rq_pair(col[v]);
        }
}

// Round cap of a PPR slot: its frontier lanes keep their residual (res = rq / (1-alpha),
// as c2g_ppr_batch leaves them) and leave the masks; dangling lanes keep theirs.
__global__ void ppr_retire_kernel(PprBatchArrays a, int b, int Q, int logW, int V, int slot, double one_m_a) {
    const int stride = gridDim.x * blockDim.x;
    const unsigned bit = 1u << (slot & 31);
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < V; v += stride) {
        const size_t wi = ((size_t)v << logW) + (size_t)(slot >> 5);
        if (a.amask[b][wi] & bit) {
            const size_t off = (size_t)v * (size_t)Q + (size_t)slot;
            a.res[off] = a.rq[b][off] / one_m_a;
            atomicAnd(a.amask[b] + wi, ~bit);
        }
        if (a.dmask[wi] & bit) atomicAnd(a.dmask + wi, ~bit);
    }
}

enum SlotState : int8_t { kFree = 0, kRunning = 1, kFinished = 2 };

}  // namespace

// A query's state outside its session, in device memory of the graph's device.
struct c2g_snapshot {
    int kind = 0;
    int32_t V = 0;
    int32_t source = 0;
    int32_t rounds = 0;   // rounds run so far (PPR: counts toward the cap)
    float alpha = 0.f, rmax = 0.f;  // PPR: the push it belongs to
    void* col4 = nullptr;       // SSSP distances (int32) / PPR pr (float)
    double* res = nullptr;      // PPR residuals
    double* rq = nullptr;       // PPR pushed residuals of the frontier lanes
    unsigned* bits_a = nullptr;  // SSSP: next-round lanes; PPR: frontier lanes with out-edges
    unsigned* bits_d = nullptr;  // PPR: dangling lanes
    int device = 0;
    ~c2g_snapshot() {
        for (void* p : {col4, (void*)res, (void*)rq, (void*)bits_a, (void*)bits_d})
            if (p) cudaFree(p);
    }
};

struct c2g_session {
    c2g_graph* g = nullptr;  // a view with its own stream and workspace
    int kind = 0;
    int Q = 0, logW = 0;
    c2g_ppr_params prm{};
    int cur = 1;  // PPR: the round the state at rest belongs to (its parity picks the buffers)
    int* dist = nullptr;
    unsigned* mask = nullptr;
    PprBatchArrays pa{};
    std::vector<int8_t> state;
    std::vector<int32_t> rounds, source, flags;
    std::vector<int2> joins;                          // (slot, source), applied at the next step
    std::vector<std::pair<int, c2g_snapshot*>> restores;  // resumed snapshots, applied at the next step
    int2* d_joins = nullptr;
    unsigned* d_active = nullptr;
    void* d_stage = nullptr;  // V floats: host read-outs from pageable memory
    std::mutex mu;
};

namespace {

int launch_blocks(const c2g_graph* g) { return g->num_sms * 8; }

void* mapped_or_null(void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

bool is_device(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Joins and restores wait on the host until the next step; this applies them.
int apply_pending(c2g_session* s) {
    c2g_graph* g = s->g;
    const int V = g->V;
    const int n = (int)s->joins.size();
    if (n) {
        C2G_CUDA(cudaMemcpyAsync(s->d_joins, s->joins.data(), sizeof(int2) * (size_t)n, cudaMemcpyHostToDevice,
                                 g->stream));
        const bool ppr = s->kind == C2G_REQ_PPR;
        join_cols_kernel<<<launch_blocks(g), 256, 0, g->stream>>>(ppr ? nullptr : s->dist, ppr ? s->pa.pr : nullptr,
                                                                  ppr ? s->pa.res : nullptr, s->Q, V, s->d_joins, n);
        if (ppr)
            ppr_join_src_kernel<<<(n + 127) / 128, 128, 0, g->stream>>>(s->pa, s->cur & 1, s->Q, s->logW, g->row,
                                                                       s->d_joins, n, s->prm.alpha, s->prm.r0,
                                                                       s->prm.pr0);
        else
            sssp_join_src_kernel<<<(n + 127) / 128, 128, 0, g->stream>>>(s->dist, s->mask, s->Q, s->logW, s->d_joins,
                                                                        n);
        C2G_CUDA(cudaGetLastError());
        C2G_CUDA(cudaStreamSynchronize(g->stream));  // the host join list is reused
        s->joins.clear();
    }
    for (auto& r : s->restores) {
        const int slot = r.first;
        c2g_snapshot* sn = r.second;
        const int bl = launch_blocks(g);
        if (s->kind == C2G_REQ_SSSP) {
            scatter_col_kernel<int><<<bl, 256, 0, g->stream>>>(s->dist, s->Q, V, slot, static_cast<int*>(sn->col4));
            restore_bits_kernel<<<bl, 256, 0, g->stream>>>(s->mask, s->logW, V, slot, sn->bits_a);
        } else {
            const int b = s->cur & 1;
            scatter_col_kernel<float><<<bl, 256, 0, g->stream>>>(s->pa.pr, s->Q, V, slot, static_cast<float*>(sn->col4));
            scatter_col_kernel<double><<<bl, 256, 0, g->stream>>>(s->pa.res, s->Q, V, slot, sn->res);
            scatter_rq_kernel<<<bl, 256, 0, g->stream>>>(s->pa.rq[b], s->pa.rqf[b], s->Q, V, slot, sn->rq, sn->bits_a);
            restore_bits_kernel<<<bl, 256, 0, g->stream>>>(s->pa.amask[b], s->logW, V, slot, sn->bits_a);
            restore_bits_kernel<<<bl, 256, 0, g->stream>>>(s->pa.dmask, s->logW, V, slot, sn->bits_d);
        }
        C2G_CUDA(cudaGetLastError());
        C2G_CUDA(cudaStreamSynchronize(g->stream));
        delete sn;
    }
    s->restores.clear();
    return C2G_OK;
}

int free_slot(c2g_session* s) {
    for (int i = 0; i < s->Q; ++i)
        if (s->state[i] == kFree) return i;
    return -1;
}

// Lanes still active (per query word) in the state at rest.
int scan_active(c2g_session* s, std::vector<unsigned>& act) {
    c2g_graph* g = s->g;
    const int W = s->Q / 32;
    const size_t n = (size_t)g->V * (size_t)W;
    C2G_CUDA(cudaMemsetAsync(s->d_active, 0, sizeof(unsigned) * (size_t)W, g->stream));
    if (s->kind == C2G_REQ_SSSP)
        active_scan_kernel<<<launch_blocks(g), 256, 0, g->stream>>>(s->mask, nullptr, n, W, s->d_active);
    else
        active_scan_kernel<<<launch_blocks(g), 256, 0, g->stream>>>(s->pa.amask[s->cur & 1], s->pa.dmask, n, W,
                                                                    s->d_active);
    C2G_CUDA(cudaGetLastError());
    act.assign((size_t)W, 0u);
    C2G_CUDA(cudaMemcpyAsync(act.data(), s->d_active, sizeof(unsigned) * (size_t)W, cudaMemcpyDeviceToHost, g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    return C2G_OK;
}

}  // namespace

extern "C" {

int c2g_session_create(c2g_graph* g, int kind, int32_t slots, const c2g_ppr_params* params, c2g_session** out) {
    if (!g || !out) return fail(C2G_ERR_ARG, "NULL argument");
    *out = nullptr;
    if (kind != C2G_REQ_SSSP && kind != C2G_REQ_PPR) return fail(C2G_ERR_ARG, "session kind must be SSSP or PPR");
    if (slots < 1 || slots > 1024) return fail(C2G_ERR_ARG, "slots must be in [1, 1024]");
    if (kind == C2G_REQ_PPR) {
        if (!params) return fail(C2G_ERR_ARG, "PPR session needs parameters");
        if (params->seeded) return fail(C2G_ERR_UNSUPPORTED, "sessions run the base-mode push (seeded = 0)");
        if (!(params->alpha > 0.f && params->alpha < 1.f) || !(params->rmax >= 0.f) || params->max_iter < 1)
            return fail(C2G_ERR_ARG, "bad PPR parameters");
    }
    c2g_session* s = new c2g_session();
    s->kind = kind;
    if (params) s->prm = *params;
    s->Q = 32;
    while (s->Q < slots) {
        s->Q <<= 1;
        ++s->logW;
    }
    int rc = C2G_OK;
    if (kind == C2G_REQ_PPR && g->adj_f && g->ppr_cfg.batch_pull_ratio >= 0.f && !g->borrowed) {
        // pull rounds read the base graph's reverse CSR; the view takes it as it is now
        std::lock_guard<std::mutex> lk(g->mu);
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(g->device);
        rc = ppr_pull_prepare(g);
        if (prev >= 0) cudaSetDevice(prev);
    }
    if (!rc) rc = graph_view(g, &s->g);
    if (!rc) {
        std::lock_guard<std::mutex> lk(s->g->mu);
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(g->device);
        rc = kind == C2G_REQ_SSSP ? sssp_batch_reserve(s->g, s->Q, &s->dist, &s->mask)
                                  : ppr_batch_reserve(s->g, s->Q, &s->pa);
        if (!rc && cudaMalloc(&s->d_joins, sizeof(int2) * (size_t)s->Q) != cudaSuccess)
            rc = fail(C2G_ERR_OOM, "session: join list");
        if (!rc && cudaMalloc(&s->d_active, sizeof(unsigned) * (size_t)(s->Q / 32)) != cudaSuccess)
            rc = fail(C2G_ERR_OOM, "session: activity words");
        if (!rc && cudaMalloc(&s->d_stage, sizeof(float) * (size_t)(g->V ? g->V : 1)) != cudaSuccess)
            rc = fail(C2G_ERR_OOM, "session: staging");
        if (prev >= 0) cudaSetDevice(prev);
    }
    if (rc) {
        c2g_session_free(s);
        return rc;
    }
    s->state.assign((size_t)s->Q, kFree);
    for (int i = slots; i < s->Q; ++i) s->state[i] = -1;  // beyond the requested slots: never used
    s->rounds.assign((size_t)s->Q, 0);
    s->source.assign((size_t)s->Q, -1);
    s->flags.assign((size_t)s->Q, 0);
    *out = s;
    return C2G_OK;
}

int c2g_session_admit(c2g_session* s, int32_t source, int32_t* slot) {
    if (!s || !slot) return fail(C2G_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (source < 0 || source >= s->g->V) return fail(C2G_ERR_RANGE, "source %d out of range [0,%d)", source, s->g->V);
    const int i = free_slot(s);
    if (i < 0) return fail(C2G_ERR_OVERFLOW, "session: no free slot");
    s->state[i] = kRunning;
    s->rounds[i] = 0;
    s->source[i] = source;
    s->flags[i] = 0;
    s->joins.push_back(make_int2(i, source));
    *slot = i;
    return C2G_OK;
}

int c2g_session_step(c2g_session* s, int32_t rounds, int32_t* finished, int32_t cap, int32_t* n_finished,
                     c2g_stats* stats) {
    if (!s || !n_finished || (cap > 0 && !finished)) return fail(C2G_ERR_ARG, "NULL argument");
    if (rounds < 1) return fail(C2G_ERR_ARG, "rounds must be >= 1");
    std::lock_guard<std::mutex> lk(s->mu);
    c2g_graph* g = s->g;
    std::lock_guard<std::mutex> glk(g->mu);
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    struct Restore {
        int d;
        ~Restore() {
            if (d >= 0) cudaSetDevice(d);
        }
    } restore_dev{prev};
    *n_finished = 0;
    if (stats) std::memset(stats, 0, sizeof(*stats));
    int rc;
    if ((rc = apply_pending(s))) return rc;
    int running = 0;
    int room = rounds;
    for (int i = 0; i < s->Q; ++i)
        if (s->state[i] == kRunning) {
            ++running;
            if (s->kind == C2G_REQ_PPR) room = std::min(room, s->prm.max_iter - s->rounds[i]);
        }
    int iters = 0;
    if (running && room > 0) {
        float ms = 0.f;
        long long counters[2] = {0, 0};
        TraversalCtl ctl;
        rc = s->kind == C2G_REQ_SSSP ? sssp_batch_epoch(g, s->Q, room, &ms, counters, &ctl)
                                     : ppr_batch_epoch(g, s->Q, s->prm, s->cur, room, &ms, counters, &ctl);
        if (rc) return rc;
        if (ctl.flags & (C2G_FLAG_BARRIER_TIMEOUT | C2G_FLAG_QUEUE_OVERFLOW | C2G_FLAG_BOUNDS))
            return fail(ctl.flags & C2G_FLAG_BARRIER_TIMEOUT ? C2G_ERR_TIMEOUT : C2G_ERR_OVERFLOW,
                        "session epoch failed (status flags 0x%x)", ctl.flags);
        iters = ctl.iterations;
        if (s->kind == C2G_REQ_PPR) s->cur += iters;
        if (stats) {
            stats->iterations = iters;
            stats->vertices_popped = ctl.popped;
            stats->edges_relaxed = counters[0];
            stats->touched = ctl.touched;
            stats->device_ms = ms;
            stats->status_flags = ctl.flags;
        }
    }
    for (int i = 0; i < s->Q; ++i)
        if (s->state[i] == kRunning) s->rounds[i] += iters;
    std::vector<unsigned> act;
    if ((rc = scan_active(s, act))) return rc;
    int nf = 0;
    for (int i = 0; i < s->Q; ++i) {
        if (s->state[i] != kRunning) continue;
        bool done = !((act[(size_t)(i >> 5)] >> (i & 31)) & 1u);
        if (!done && s->kind == C2G_REQ_PPR && s->rounds[i] >= s->prm.max_iter) {
            ppr_retire_kernel<<<launch_blocks(g), 256, 0, g->stream>>>(s->pa, s->cur & 1, s->Q, s->logW, g->V, i,
                                                                       1.0 - (double)s->prm.alpha);
            C2G_CUDA(cudaGetLastError());
            C2G_CUDA(cudaStreamSynchronize(g->stream));
            s->flags[i] |= C2G_FLAG_ITER_CAP;
            done = true;
        }
        if (done) {
            s->state[i] = kFinished;
            if (nf < cap) finished[nf] = i;
            ++nf;
        }
    }
    *n_finished = nf;
    return C2G_OK;
}

int c2g_session_read(c2g_session* s, int32_t slot, void* out, float* res_out, int on_device, c2g_stats* stats) {
    if (!s || !out) return fail(C2G_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (slot < 0 || slot >= s->Q || s->state[slot] != kFinished)
        return fail(C2G_ERR_ARG, "slot %d holds no finished query", slot);
    c2g_graph* g = s->g;
    std::lock_guard<std::mutex> glk(g->mu);
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    const int V = g->V;
    cudaError_t e = cudaSuccess;
    void* outs[2] = {out, res_out};
    for (int k = 0; k < 2 && e == cudaSuccess; ++k) {
        if (!outs[k] || (k == 1 && s->kind != C2G_REQ_PPR)) continue;
        if (on_device && !is_device(outs[k])) {
            e = cudaErrorInvalidValue;
            break;
        }
        void* mapped = on_device ? nullptr : mapped_or_null(outs[k]);
        void* dst = on_device ? outs[k] : (mapped ? mapped : s->d_stage);
        const int bl = launch_blocks(g);
        if (s->kind == C2G_REQ_SSSP)
            gather_col_kernel<int, int><<<bl, 256, 0, g->stream>>>(s->dist, s->Q, V, slot, static_cast<int*>(dst));
        else if (k == 0)
            gather_col_kernel<float, float><<<bl, 256, 0, g->stream>>>(s->pa.pr, s->Q, V, slot, static_cast<float*>(dst));
        else
            gather_col_kernel<double, float><<<bl, 256, 0, g->stream>>>(s->pa.res, s->Q, V, slot,
                                                                        static_cast<float*>(dst));
        e = cudaGetLastError();
        if (e == cudaSuccess && !on_device && !mapped)
            e = cudaMemcpyAsync(outs[k], s->d_stage, sizeof(float) * (size_t)V, cudaMemcpyDeviceToHost, g->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    }
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) return fail(C2G_ERR_CUDA, "session read: %s", cudaGetErrorString(e));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->source = s->source[slot];
        stats->iterations = s->rounds[slot];
        stats->status_flags = s->flags[slot];
    }
    s->state[slot] = kFree;
    return C2G_OK;
}

int c2g_session_evict(c2g_session* s, int32_t slot, c2g_snapshot** out) {
    if (!s || !out) return fail(C2G_ERR_ARG, "NULL argument");
    *out = nullptr;
    std::lock_guard<std::mutex> lk(s->mu);
    if (slot < 0 || slot >= s->Q || s->state[slot] != kRunning)
        return fail(C2G_ERR_ARG, "slot %d holds no running query", slot);
    for (const int2& j : s->joins)
        if (j.x == slot) return fail(C2G_ERR_ARG, "slot %d has not started yet (it joins at the next step)", slot);
    for (const auto& r : s->restores)
        if (r.first == slot) return fail(C2G_ERR_ARG, "slot %d resumes at the next step", slot);
    c2g_graph* g = s->g;
    std::lock_guard<std::mutex> glk(g->mu);
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    const int V = g->V;
    const size_t nb = (size_t)((V + 31) / 32);
    c2g_snapshot* sn = new c2g_snapshot();
    sn->kind = s->kind;
    sn->V = V;
    sn->source = s->source[slot];
    sn->rounds = s->rounds[slot];
    sn->device = g->device;
    sn->alpha = s->prm.alpha;
    sn->rmax = s->prm.rmax;
    cudaError_t e = cudaMalloc(&sn->col4, sizeof(int32_t) * (size_t)V);
    if (e == cudaSuccess) e = cudaMalloc(&sn->bits_a, sizeof(unsigned) * nb);
    if (e == cudaSuccess && s->kind == C2G_REQ_PPR) {
        e = cudaMalloc(&sn->res, sizeof(double) * (size_t)V);
        if (e == cudaSuccess) e = cudaMalloc(&sn->rq, sizeof(double) * (size_t)V);
        if (e == cudaSuccess) e = cudaMalloc(&sn->bits_d, sizeof(unsigned) * nb);
    }
    const int bl = launch_blocks(g);
    if (e == cudaSuccess) {
        if (s->kind == C2G_REQ_SSSP) {
            gather_col_kernel<int, int><<<bl, 256, 0, g->stream>>>(s->dist, s->Q, V, slot, static_cast<int*>(sn->col4));
            snap_bits_kernel<<<bl, 256, 0, g->stream>>>(s->mask, s->logW, V, slot, 1, sn->bits_a);
        } else {
            const int b = s->cur & 1;
            gather_col_kernel<float, float><<<bl, 256, 0, g->stream>>>(s->pa.pr, s->Q, V, slot,
                                                                       static_cast<float*>(sn->col4));
            gather_col_kernel<double, double><<<bl, 256, 0, g->stream>>>(s->pa.res, s->Q, V, slot, sn->res);
            gather_col_kernel<double, double><<<bl, 256, 0, g->stream>>>(s->pa.rq[b], s->Q, V, slot, sn->rq);
            snap_bits_kernel<<<bl, 256, 0, g->stream>>>(s->pa.amask[b], s->logW, V, slot, 1, sn->bits_a);
            snap_bits_kernel<<<bl, 256, 0, g->stream>>>(s->pa.dmask, s->logW, V, slot, 1, sn->bits_d);
        }
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) {
        delete sn;
        return fail(e == cudaErrorMemoryAllocation ? C2G_ERR_OOM : C2G_ERR_CUDA, "session evict: %s",
                    cudaGetErrorString(e));
    }
    s->state[slot] = kFree;
    *out = sn;
    return C2G_OK;
}

int c2g_session_resume(c2g_session* s, c2g_snapshot* snap, int32_t* slot) {
    if (!s || !snap || !slot) return fail(C2G_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (snap->kind != s->kind || snap->V != s->g->V || snap->device != s->g->device)
        return fail(C2G_ERR_ARG, "snapshot belongs to another kind of session or graph");
    if (s->kind == C2G_REQ_PPR && (snap->alpha != s->prm.alpha || snap->rmax != s->prm.rmax))
        return fail(C2G_ERR_ARG, "snapshot belongs to a push with other parameters (alpha, rmax)");
    if (s->kind == C2G_REQ_PPR && snap->rounds > s->prm.max_iter)
        return fail(C2G_ERR_ARG, "snapshot has run past this session's round cap");
    const int i = free_slot(s);
    if (i < 0) return fail(C2G_ERR_OVERFLOW, "session: no free slot");
    s->state[i] = kRunning;
    s->rounds[i] = snap->rounds;
    s->source[i] = snap->source;
    s->flags[i] = 0;
    s->restores.emplace_back(i, snap);
    *slot = i;
    return C2G_OK;
}

void c2g_snapshot_free(c2g_snapshot* snap) { delete snap; }

}  // extern "C"

// The share of the SMs a session's launches take (the serving loop runs three kinds side
// by side, each on a third, so their persistent kernels are co-resident).
void c2g::session_set_grid_share(c2g_session* s, float share) {
    std::lock_guard<std::mutex> lk(s->mu);
    s->g->grid_scale = share;
}

extern "C" {

int c2g_session_slot(c2g_session* s, int32_t slot, int32_t* state, int32_t* source, int32_t* rounds) {
    if (!s) return fail(C2G_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(s->mu);
    if (slot < 0 || slot >= s->Q) return fail(C2G_ERR_RANGE, "slot %d out of range", slot);
    if (state) *state = s->state[slot] < 0 ? 0 : s->state[slot];
    if (source) *source = s->source[slot];
    if (rounds) *rounds = s->rounds[slot];
    return C2G_OK;
}

void c2g_session_free(c2g_session* s) {
    if (!s) return;
    for (auto& r : s->restores) delete r.second;
    if (s->g) {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(s->g->device);
        for (void* p : {(void*)s->d_joins, (void*)s->d_active, s->d_stage})
            if (p) cudaFree(p);
        graph_free_view(s->g);
        if (prev >= 0) cudaSetDevice(prev);
    }
    delete s;
}

}  // extern "C"
