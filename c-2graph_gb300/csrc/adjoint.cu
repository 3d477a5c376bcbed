// PPR adjoint for sm_103a: gradient of L = sum_{t in T} pi_s(t) with respect to every
// flist edge weight.
//
// With the reference's convention (pr += alpha*r, push (1-alpha)*r*w,
// src/ppr/base/Main.cu:146-150 and :288), pi = alpha * (I - (1-alpha) P^T)^{-1} e_s for
// P[u][v] = w(u,v).  Then
//     dL/dw(u,v) = (1-alpha) * pi(u) * lambda(v),  lambda = (I - (1-alpha) P)^{-1} 1_T.
// lambda is the fixed point of lambda(u) = 1_T(u) + (1-alpha) sum_v w(u,v) lambda(v),
// computed by a transposed push: the same BSP push kernel, run on the reverse CSR
// (in-edges carrying w(u,v)) from the target set, absorbing 1*r instead of alpha*r.
// The gradient pass reads each forward edge once: 12 bytes per edge + 8 per vertex.
#include <algorithm>
#include <cstring>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

namespace c2g {

// In-degree count over the forward CSR.
__global__ void count_in_kernel(const int2* __restrict__ adj, long long E, int* __restrict__ indeg) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride)
        atomicAdd(indeg + adj[e].x, 1);
}

// Scatter every forward edge u->v (weight bits) into v's in-edge row as (u, weight).
__global__ void scatter_in_kernel(const int* __restrict__ row, const int2* __restrict__ adj, int V,
                                  int* __restrict__ cursor, int2* __restrict__ adj_r) {
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int nwarps = (gridDim.x * blockDim.x) >> 5;
    for (int u = warp; u < V; u += nwarps) {
        for (int e = row[u] + lane; e < row[u + 1]; e += 32) {
            const int2 ew = adj[e];
            const int pos = atomicAdd(cursor + ew.x, 1);
            adj_r[pos] = make_int2(u, ew.y);
        }
    }
}

// grad[e] = c * pi[u] * lambda[col[e]] for every forward edge e = (u -> col[e]).  Warps
// take tiles of 2^kPullTileLog edges; a tile's first owner comes from the forward tile
// markers (one load), the next 32 owners' row bounds and pi values one per lane, and each
// edge's owner from a shuffle search.  Edges are read 32 at a time, kGradUnroll batches in
// flight, so the lambda gathers of a warp overlap.
constexpr int kGradUnroll = 4;

__global__ void adjoint_grad_kernel(const int* __restrict__ row, const int2* __restrict__ adj,
                                    const int* __restrict__ mark, int V, unsigned E, const float* __restrict__ pi,
                                    const float* __restrict__ lam, float c, float* __restrict__ grad,
                                    int* __restrict__ flags) {
    const int lane = threadIdx.x & 31;
    const unsigned warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const unsigned nwarps = (gridDim.x * blockDim.x) >> 5;
    const unsigned tw = 1u << kPullTileLog;
    const unsigned ntiles = (E + tw - 1) >> kPullTileLog;
    for (unsigned t = warp; t < ntiles; t += nwarps) {
        unsigned e0 = t << kPullTileLog;
        const unsigned e1 = min(e0 + tw, E);
        unsigned o = (unsigned)__ldg(mark + t);
        while (e0 < e1) {
            const unsigned j = o + (unsigned)lane;
            unsigned base = 0x7fffffffu, endv = 0xffffffffu;
            float pj = 0.f;
            if (j < (unsigned)V) {
                base = (unsigned)__ldg(row + j);
                endv = (unsigned)__ldg(row + j + 1);
                pj = __ldg(pi + j);
            }
            if (o >= (unsigned)V || (unsigned)__shfl_sync(kFull, (int)base, 0) > e0) {
                if (lane == 0) atomicOr(flags, C2G_FLAG_BOUNDS);
                break;
            }
            const unsigned seg_end = min(e1, (unsigned)__shfl_sync(kFull, endv, 31));
            if (seg_end <= e0) {  // 32 owners without edges here (o grows to V at most)
                o += 32;
                continue;
            }
            for (unsigned eb = e0; eb < seg_end; eb += 32u * kGradUnroll) {
                int2 ew[kGradUnroll];
                float pk[kGradUnroll];
#pragma unroll
                for (int u = 0; u < kGradUnroll; ++u) {
                    const unsigned e = eb + (unsigned)lane + 32u * u;
                    pk[u] = __shfl_sync(kFull, pj, owner_lane(base, e));
                    ew[u] = e < seg_end ? __ldg(adj + e) : make_int2(0, 0);
                }
#pragma unroll
                for (int u = 0; u < kGradUnroll; ++u) {
                    const unsigned e = eb + (unsigned)lane + 32u * u;
                    if (e < seg_end) grad[e] = c * pk[u] * __ldg(lam + ew[u].x);
                }
            }
            e0 = seg_end;
            o += 32;
        }
    }
}

// Reverse CSR of the float-weighted graph (in-edges carrying w(u,v)), built once.
int build_reverse_graph(c2g_graph* g) {
    if (g->adj_r) return C2G_OK;
    const int2* fwd = g->adj_f ? g->adj_f : g->adj_w;  // float weights when the graph has them
    if (!fwd) return fail(C2G_ERR_UNSUPPORTED, "graph has no edge weights");
    const size_t V = (size_t)g->V, E = (size_t)g->E;
    int* indeg = nullptr;
    C2G_CUDA(cudaMalloc(&g->row_r, sizeof(int) * (V + 1)));
    C2G_CUDA(cudaMalloc(&g->adj_r, sizeof(int2) * (E ? E : 1)));
    C2G_CUDA(cudaMalloc(&indeg, sizeof(int) * (V ? V : 1)));
    cudaError_t e = cudaMemsetAsync(indeg, 0, sizeof(int) * V, g->stream);
    if (e == cudaSuccess && E) {
        count_in_kernel<<<g->num_sms * 4, 256, 0, g->stream>>>(fwd, (long long)E, indeg);
        e = cudaGetLastError();
    }
    std::vector<int> h(V + 1, 0);
    if (e == cudaSuccess) e = cudaMemcpyAsync(h.data() + 1, indeg, sizeof(int) * V, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    for (size_t v = 0; v < V; ++v) h[v + 1] += h[v];
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(g->row_r, h.data(), sizeof(int) * (V + 1), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(indeg, h.data(), sizeof(int) * V, cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess && E) {
        scatter_in_kernel<<<g->num_sms * 4, 256, 0, g->stream>>>(g->row, fwd, g->V, indeg, g->adj_r);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(indeg);
    C2G_CUDA(e);
    int rc = build_markers(g, g->row_r, &g->mark_r);
    if (!rc) rc = build_markers(g, g->row, &g->mark_f);
    return rc;
}

// The in-edges with int32 weights for the batched SSSP's pull rounds, in row_r's rows: adj_r
// itself when the graph has no float weights, else a second scatter of adj_w (the order
// within a row may differ from adj_r's; a minimum does not depend on it).
int build_reverse_int(c2g_graph* g) {
    if (g->adj_rw) return C2G_OK;
    if (!g->adj_w) return fail(C2G_ERR_UNSUPPORTED, "graph has no int32 weights (wlist)");
    int rc = build_reverse_graph(g);
    if (rc) return rc;
    if (!g->adj_f) {
        g->adj_rw = g->adj_r;
        return C2G_OK;
    }
    const size_t V = (size_t)g->V, E = (size_t)g->E;
    int* cursor = nullptr;
    C2G_CUDA(cudaMalloc(&g->adj_rw, sizeof(int2) * (E ? E : 1)));
    C2G_CUDA(cudaMalloc(&cursor, sizeof(int) * (V ? V : 1)));
    cudaError_t e = cudaMemcpyAsync(cursor, g->row_r, sizeof(int) * V, cudaMemcpyDeviceToDevice, g->stream);
    if (e == cudaSuccess && E) {
        scatter_in_kernel<<<g->num_sms * 4, 256, 0, g->stream>>>(g->row, g->adj_w, g->V, cursor, g->adj_rw);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(cursor);
    C2G_CUDA(e);
    return C2G_OK;
}

void adjoint_free(c2g_graph* g) {
    if (g->adj_rw && g->adj_rw != g->adj_r) cudaFree(g->adj_rw);
    g->adj_rw = nullptr;
    void* ptrs[] = {g->row_r, g->adj_r, g->mark_r, g->mark_f};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    g->wstat_valid = false;
    g->row_r = nullptr;
    g->adj_r = nullptr;
    g->mark_r = nullptr;
    g->mark_f = nullptr;
}

int set_float_weights(c2g_graph* g, const float* w, int on_device);

}  // namespace c2g

using namespace c2g;

extern "C" int c2g_ppr_adjoint(c2g_graph* g, int32_t source, const c2g_ppr_params* params, int32_t n_targets,
                               const int32_t* targets, float rmax_backward, float* grad, float* pi_out,
                               float* lambda_out, double* loss, int on_device, c2g_stats* stats) {
    if (!g || !params || !targets || !grad) return fail(C2G_ERR_ARG, "NULL argument");
    if (source < 0 || source >= g->V) return fail(C2G_ERR_RANGE, "source %d out of range [0,%d)", source, g->V);
    if (n_targets < 1) return fail(C2G_ERR_ARG, "need at least one target");
    if (!(params->alpha > 0.f && params->alpha < 1.f)) return fail(C2G_ERR_ARG, "alpha must be in (0,1)");
    if (params->seeded) return fail(C2G_ERR_UNSUPPORTED, "the adjoint differentiates the base push");
    if (!(rmax_backward >= 0.f)) return fail(C2G_ERR_ARG, "rmax_backward must be >= 0");
    if (!g->adj_f) return fail(C2G_ERR_UNSUPPORTED, "graph has no float weights (flist)");
    // distinct targets, each with its multiplicity as the initial residual
    std::vector<int32_t> tv;
    std::vector<float> tr;
    {
        std::vector<int32_t> sorted(targets, targets + n_targets);
        for (int32_t t : sorted)
            if (t < 0 || t >= g->V) return fail(C2G_ERR_RANGE, "target %d out of range", t);
        std::sort(sorted.begin(), sorted.end());
        for (size_t i = 0; i < sorted.size(); ++i) {
            if (tv.empty() || tv.back() != sorted[i]) {
                tv.push_back(sorted[i]);
                tr.push_back(1.0f);
            } else {
                tr.back() += 1.0f;
            }
        }
    }
    std::lock_guard<std::mutex> lk(g->mu);
    struct Scope {
        int prev = -1;
        explicit Scope(int d) {
            cudaGetDevice(&prev);
            cudaSetDevice(d);
        }
        ~Scope() {
            if (prev >= 0) cudaSetDevice(prev);
        }
    } scope(g->device);
    int rc = build_reverse_graph(g);
    if (rc) return rc;
    const size_t V = (size_t)g->V, E = (size_t)g->E;
    float *pi = nullptr, *lam = nullptr, *dgrad = nullptr, *dtr = nullptr;
    int32_t* dtv = nullptr;
    C2G_CUDA(cudaMalloc(&pi, sizeof(float) * V));
    C2G_CUDA(cudaMalloc(&lam, sizeof(float) * V));
    C2G_CUDA(cudaMalloc(&dtv, sizeof(int32_t) * tv.size()));
    C2G_CUDA(cudaMalloc(&dtr, sizeof(float) * tr.size()));
    dgrad = on_device ? grad : nullptr;
    if (!dgrad) C2G_CUDA(cudaMalloc(&dgrad, sizeof(float) * (E ? E : 1)));
    auto cleanup = [&]() {
        cudaFree(pi);
        cudaFree(lam);
        cudaFree(dtv);
        cudaFree(dtr);
        if (!on_device) cudaFree(dgrad);
    };
    float ms_f = 0.f, ms_b = 0.f, ms_g = 0.f;
    TraversalCtl cf, cb;
    cudaError_t e = cudaMemcpyAsync(dtv, tv.data(), sizeof(int32_t) * tv.size(), cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(dtr, tr.data(), sizeof(float) * tr.size(), cudaMemcpyHostToDevice, g->stream);
    if (e != cudaSuccess) {
        cleanup();
        C2G_CUDA(e);
    }
    // forward: pi
    c2g_ppr_params fp = *params;
    fp.r0 = 1.0f;
    fp.pr0 = fp.alpha;
    rc = ppr_launch_view(g, g->row, g->adj_f, g->row_r, g->adj_r, g->mark_r, source, fp, fp.alpha, 0, nullptr,
                         nullptr, nullptr, nullptr, 0, pi, nullptr, &ms_f);
    if (!rc && (cudaMemcpyAsync(&cf, g->ppr.ctl, sizeof(cf), cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
                cudaStreamSynchronize(g->stream) != cudaSuccess))
        rc = fail(C2G_ERR_CUDA, "adjoint: reading the forward push status failed");
    // backward: lambda, transposed push from the targets, absorbing the whole residual
    c2g_ppr_params bp = *params;
    bp.rmax = rmax_backward;
    if (!rc)
        rc = ppr_launch_view(g, g->row_r, g->adj_r, g->row, g->adj_f, g->mark_f, tv[0], bp, 1.0f, (int32_t)tv.size(),
                             dtv, dtr, nullptr, nullptr, 0, lam, nullptr, &ms_b);
    if (!rc && (cudaMemcpyAsync(&cb, g->ppr.ctl, sizeof(cb), cudaMemcpyDeviceToHost, g->stream) != cudaSuccess ||
                cudaStreamSynchronize(g->stream) != cudaSuccess))
        rc = fail(C2G_ERR_CUDA, "adjoint: reading the backward push status failed");
    if (rc) {
        cleanup();
        return rc;
    }
    if ((cf.flags | cb.flags) & (C2G_FLAG_BARRIER_TIMEOUT | C2G_FLAG_QUEUE_OVERFLOW | C2G_FLAG_BOUNDS)) {
        cleanup();
        return fail(C2G_ERR_OVERFLOW, "adjoint push reported device errors (flags %d/%d)", cf.flags, cb.flags);
    }
    // gradient pass
    cudaEventRecord(g->ev0, g->stream);
    if (E)
        adjoint_grad_kernel<<<g->num_sms * 8, 256, 0, g->stream>>>(g->row, g->adj_f, g->mark_f, g->V, (unsigned)E, pi,
                                                                   lam, 1.0f - params->alpha, dgrad,
                                                                   &g->ppr.ctl->flags);
    cudaEventRecord(g->ev1, g->stream);
    e = cudaGetLastError();
    if (e == cudaSuccess && !on_device)
        e = cudaMemcpyAsync(grad, dgrad, sizeof(float) * E, cudaMemcpyDeviceToHost, g->stream);
    std::vector<float> hpi(V);
    if (e == cudaSuccess) e = cudaMemcpyAsync(hpi.data(), pi, sizeof(float) * V, cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess && pi_out)
        e = cudaMemcpyAsync(pi_out, pi, sizeof(float) * V, on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost,
                            g->stream);
    if (e == cudaSuccess && lambda_out)
        e = cudaMemcpyAsync(lambda_out, lam, sizeof(float) * V,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, g->stream);
    int gflags = 0;  // the gradient pass's bounds checks report into the push's control block
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(&gflags, &g->ppr.ctl->flags, sizeof(int), cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) cudaEventElapsedTime(&ms_g, g->ev0, g->ev1);
    cleanup();
    C2G_CUDA(e);
    if (gflags & C2G_FLAG_BOUNDS) return fail(C2G_ERR_OVERFLOW, "adjoint gradient pass: device index check failed");
    if (loss) {
        double L = 0.0;
        for (int32_t t = 0; t < n_targets; ++t) L += (double)hpi[targets[t]];
        *loss = L;
    }
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->source = source;
        stats->iterations = cf.iterations + cb.iterations;
        stats->vertices_popped = cf.popped + cb.popped;
        stats->edges_relaxed = cf.relaxed + cb.relaxed;
        stats->touched = cf.touched + cb.touched;
        stats->n_seeds = (int64_t)tv.size();
        stats->device_ms = ms_f + ms_b + ms_g;
        stats->status_flags = cf.flags | cb.flags;
        // two pushes (12V + 20F + 12R each) + the gradient pass (12E + 8V)
        stats->alg_bytes = 24.0 * V + 20.0 * (double)(cf.popped + cb.popped) + 12.0 * (double)(cf.relaxed + cb.relaxed) +
                           12.0 * (double)E + 8.0 * (double)V;
    }
    return C2G_OK;
}

extern "C" int c2g_graph_set_weights(c2g_graph* g, const float* flist, int on_device) {
    if (!g || !flist) return fail(C2G_ERR_ARG, "NULL argument");
    std::lock_guard<std::mutex> lk(g->mu);
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    const int rc = set_float_weights(g, flist, on_device);
    if (prev >= 0) cudaSetDevice(prev);
    return rc;
}
