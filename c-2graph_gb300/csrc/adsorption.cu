// Adsorption label propagation for sm_103a.
//
// The reference's "adsorption" programs are the PPR push with a different start
// (src/adsorption/w-base/Main.cu:124-395, served here by c2g_ppr with
// c2g_ppr_default_params(g, 1, ...)); they carry no labels.  This file is the
// label-propagation form of adsorption that the serving configuration asks for:
//     Y_v <- p_inj(v) * I_v + p_cont(v) * sum_{u->v} w(u,v) * Y_u
// over L = 16 labels per query (I_v = 1 for the vertex seeding label l), iterated a
// fixed number of times from Y = I.  The abandonment share p_abnd(v) goes to the dummy
// "none" label, which is not stored.
//
// One iteration is a pull over the reverse CSR: the in-edges of all vertices form one
// range [0, E) cut into tiles of 2^kPullTileLog edges; a group of 4 lanes (each holding 4
// of the 16 labels as a float4) walks a tile from its marker's owner, its in-edges staged
// through shared memory 32 at a time (16-byte loads, read back as broadcasts: 41.98 vs
// 42.80 ms per query at scale 22 against shuffling them within the group), accumulating
// per-owner sums in registers, and writes each owner's row with a plain store when the
// owner's in-edges lie inside the tile, otherwise with atomicAdd (only owners straddling
// a tile boundary).  kAdsBatch label rows are gathered before they are used.  A vertex
// pass then applies p_inj / p_cont.
// Per iteration: (8 + 64) bytes per edge (in-edge record + source label row) and
// 64 + 64 + 12 bytes per vertex.  The iteration sequence is captured once per handle
// (and iteration count) into a CUDA graph and replayed; its buffers stay with the handle.
#include <cstring>
#include <vector>

#include "device_common.cuh"
#include "internal.h"

namespace c2g {

constexpr int kAdsL = 16;          // labels per query

constexpr int kAdsBatch = 8;      // in-edges whose label rows a group gathers at once
constexpr int kAdsMinBlocks = 3;  // launch bounds: resident 256-thread blocks per SM
constexpr int kAdsThreads = 256;
constexpr int kAdsChunk = 32;     // in-edges a group stages in shared memory at a time

__global__ void __launch_bounds__(kAdsThreads, kAdsMinBlocks) ads_edge_pass(const int* __restrict__ row_r,
                                                                            const int2* __restrict__ adj_r,
                              const int* __restrict__ mark_r, int V, unsigned E, const float4* __restrict__ Y,
                              float* __restrict__ acc) {
    const int lane = threadIdx.x & 31;
    const int part = lane & 3;                   // labels 4*part .. 4*part+3 of every row
    const int g0 = lane & ~3;                    // first lane of this 4-lane group
    const unsigned gmask = 0xfu << g0;           // the group's lanes (groups diverge)
    const unsigned ngroups = (gridDim.x * blockDim.x) >> 2;
    const unsigned tw = 1u << kPullTileLog;
    const unsigned ntiles = (E + tw - 1) >> kPullTileLog;
    // each group's staged in-edges; one pad entry per row, so that the 8 groups of a warp,
    // reading entry k of their rows at once, hit 8 different bank pairs
    __shared__ int2 staged[kAdsThreads / 4][kAdsChunk + 1];
    int2* const st = staged[threadIdx.x >> 2];
    for (unsigned t = (blockIdx.x * blockDim.x + threadIdx.x) >> 2; t < ntiles; t += ngroups) {
        const unsigned e0 = t << kPullTileLog;
        const unsigned e1 = min(e0 + tw, E);
        int v = __ldg(mark_r + t);               // owner of in-edge e0
        unsigned vend = (unsigned)__ldg(row_r + v + 1);
        bool whole = (unsigned)__ldg(row_r + v) >= e0;
        float4 s = make_float4(0.f, 0.f, 0.f, 0.f);
        for (unsigned c = e0; c < e1; c += kAdsChunk) {
            // stage the chunk: each lane loads 2 in-edges at a time (16-byte loads; c is even)
            __syncwarp(gmask);  // the previous chunk's reads are done
#pragma unroll
            for (int r = 0; r < kAdsChunk / 8; ++r) {
                const unsigned idx = c + 2u * part + 8u * r;
                int4 two = make_int4(0, 0, 0, 0);
                if (idx + 1 < e1) {
                    two = __ldg(reinterpret_cast<const int4*>(adj_r + idx));
                } else if (idx < e1) {
                    const int2 one = __ldg(adj_r + idx);
                    two.x = one.x;
                    two.y = one.y;
                }
                st[2 * part + 8 * r] = make_int2(two.x, two.y);
                st[2 * part + 8 * r + 1] = make_int2(two.z, two.w);
            }
            __syncwarp(gmask);
            const unsigned cend = min(c + kAdsChunk, e1);
            for (unsigned b = c; b < cend; b += kAdsBatch) {
                // kAdsBatch in-edges read from the stage (broadcast within the group), their
                // label rows gathered together, then consumed in order
                float4 y[kAdsBatch];
                float wt[kAdsBatch];
#pragma unroll
                for (int k = 0; k < kAdsBatch; ++k) {
                    const int2 ek = st[b - c + k];
                    wt[k] = __int_as_float(ek.y);
                    y[k] = b + k < e1 ? __ldg(Y + (size_t)ek.x * (kAdsL / 4) + part) : make_float4(0.f, 0.f, 0.f, 0.f);
                }
#pragma unroll
                for (int k = 0; k < kAdsBatch; ++k) {
                    const unsigned e = b + k;
                    if (e >= e1) break;  // group-uniform
                    while (e >= vend) {  // owner changes: write the finished owner's row part
                        float* o = acc + (size_t)v * kAdsL + 4 * part;
                        if (whole) {
                            *reinterpret_cast<float4*>(o) = s;
                        } else {
                            atomicAdd(o, s.x);
                            atomicAdd(o + 1, s.y);
                            atomicAdd(o + 2, s.z);
                            atomicAdd(o + 3, s.w);
                        }
                        s = make_float4(0.f, 0.f, 0.f, 0.f);
                        ++v;
                        whole = true;  // rows starting inside the tile
                        vend = (unsigned)__ldg(row_r + v + 1);
                    }
                    s.x = fmaf(wt[k], y[k].x, s.x);
                    s.y = fmaf(wt[k], y[k].y, s.y);
                    s.z = fmaf(wt[k], y[k].z, s.z);
                    s.w = fmaf(wt[k], y[k].w, s.w);
                }
            }
        }
        float* o = acc + (size_t)v * kAdsL + 4 * part;
        if (whole && vend <= e1) {
            *reinterpret_cast<float4*>(o) = s;
        } else {
            atomicAdd(o, s.x);
            atomicAdd(o + 1, s.y);
            atomicAdd(o + 2, s.z);
            atomicAdd(o + 3, s.w);
        }
    }
}

// Y[v][l] = p_cont(v) * acc[v][l] + (label l seeded at v ? p_inj(v) : 0); acc = 0.
__global__ void ads_vertex_pass(int V, const float* __restrict__ p_inj, const float* __restrict__ p_cont,
                                const unsigned* __restrict__ seedmask, float* __restrict__ acc, float* __restrict__ Y) {
    const size_t n = (size_t)V * kAdsL;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const size_t v = i / kAdsL;
        const int l = (int)(i % kAdsL);
        const float inj = ((seedmask[v] >> l) & 1u) ? p_inj[v] : 0.f;
        Y[i] = fmaf(p_cont[v], acc[i], inj);
        acc[i] = 0.f;
    }
}

// Y = I (seed labels), acc = 0.
__global__ void ads_init(int V, const unsigned* __restrict__ seedmask, float* __restrict__ acc, float* __restrict__ Y) {
    const size_t n = (size_t)V * kAdsL;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        Y[i] = ((seedmask[i / kAdsL] >> (i % kAdsL)) & 1u) ? 1.f : 0.f;
        acc[i] = 0.f;
    }
}

// Seed mask from the 16 seed vertices: bit l of mask[v] says label l is seeded at v.
__global__ void ads_seed_mask(const int* __restrict__ seeds, int n, unsigned* __restrict__ mask) {
    const int l = threadIdx.x;
    if (l < n) atomicOr(mask + seeds[l], 1u << l);
}

// Per-handle workspace of the label propagation, kept across calls so that a serving
// loop's adsorption requests allocate nothing after the first one (cudaMalloc and
// cudaFree synchronise the device and would stall the other kinds' batches), with the
// iteration sequence captured once into a CUDA graph and replayed.
struct AdsWork {
    float* Y = nullptr;    // [V][16]
    float* acc = nullptr;  // [V][16]
    unsigned* mask = nullptr;
    float* pi = nullptr;
    float* pc = nullptr;
    int* seeds = nullptr;  // [16]
    cudaGraphExec_t exec = nullptr;
    int iterations = -1;
};

void ads_free(c2g_graph* g) {
    AdsWork* w = reinterpret_cast<AdsWork*>(g->ads);
    if (!w) return;
    if (w->exec) cudaGraphExecDestroy(w->exec);
    void* ptrs[] = {w->Y, w->acc, w->mask, w->pi, w->pc, w->seeds};
    for (void* q : ptrs)
        if (q) cudaFree(q);
    delete w;
    g->ads = nullptr;
}

static int ads_alloc(c2g_graph* g, AdsWork** out) {
    AdsWork* w = reinterpret_cast<AdsWork*>(g->ads);
    if (!w) {
        w = new AdsWork();
        g->ads = w;
        const size_t V = g->V ? (size_t)g->V : 1;
        C2G_CUDA(cudaMalloc(&w->Y, sizeof(float) * V * kAdsL));
        C2G_CUDA(cudaMalloc(&w->acc, sizeof(float) * V * kAdsL));
        C2G_CUDA(cudaMalloc(&w->mask, sizeof(unsigned) * V));
        C2G_CUDA(cudaMalloc(&w->pi, sizeof(float) * V));
        C2G_CUDA(cudaMalloc(&w->pc, sizeof(float) * V));
        C2G_CUDA(cudaMalloc(&w->seeds, sizeof(int) * kAdsL));
    }
    *out = w;
    return C2G_OK;
}

// Capture init + `iterations` x (edge pass, vertex pass) on the handle's stream.
static int ads_capture(c2g_graph* g, AdsWork* w, int iterations) {
    if (w->exec && w->iterations == iterations) return C2G_OK;
    if (w->exec) {
        cudaGraphExecDestroy(w->exec);
        w->exec = nullptr;
    }
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal);
    if (e == cudaSuccess) {
        const int eb = g->num_sms * 8, vb = g->num_sms * 8;
        ads_init<<<vb, 256, 0, g->stream>>>(g->V, w->mask, w->acc, w->Y);
        for (int it = 0; it < iterations; ++it) {
            if (g->E)
                ads_edge_pass<<<eb, kAdsThreads, 0, g->stream>>>(g->row_r, g->adj_r, g->mark_r, g->V, (unsigned)g->E,
                                                          reinterpret_cast<const float4*>(w->Y), w->acc);
            ads_vertex_pass<<<vb, 256, 0, g->stream>>>(g->V, w->pi, w->pc, w->mask, w->acc, w->Y);
        }
        e = cudaStreamEndCapture(g->stream, &graph);
    }
    if (e == cudaSuccess) e = cudaGraphInstantiate(&w->exec, graph, 0);
    if (graph) cudaGraphDestroy(graph);
    C2G_CUDA(e);
    w->iterations = iterations;
    return C2G_OK;
}

}  // namespace c2g

using namespace c2g;

extern "C" int c2g_adsorption(c2g_graph* g, int32_t n_labels, const int32_t* seed_vertices, const float* p_inj,
                              const float* p_cont, const float* p_abnd, int32_t iterations, float* Y_out,
                              int on_device, c2g_stats* stats) {
    if (!g || !seed_vertices || !p_inj || !p_cont || !Y_out) return fail(C2G_ERR_ARG, "NULL argument");
    if (n_labels != kAdsL) return fail(C2G_ERR_UNSUPPORTED, "adsorption supports %d labels per query", kAdsL);
    if (iterations < 0) return fail(C2G_ERR_ARG, "iterations must be >= 0");
    if (!g->adj_f) return fail(C2G_ERR_UNSUPPORTED, "graph has no float weights (flist)");
    (void)p_abnd;  // the abandonment share goes to the unstored dummy label
    for (int32_t l = 0; l < n_labels; ++l)
        if (seed_vertices[l] < 0 || seed_vertices[l] >= g->V)
            return fail(C2G_ERR_RANGE, "seed vertex %d out of range", seed_vertices[l]);
    std::lock_guard<std::mutex> lk(g->mu);
    int prev = -1;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    struct Restore {
        int d;
        ~Restore() {
            if (d >= 0) cudaSetDevice(d);
        }
    } restore{prev};
    int rc = build_reverse_graph(g);
    if (rc) return rc;
    AdsWork* w = nullptr;
    if ((rc = ads_alloc(g, &w))) return rc;
    const size_t V = (size_t)g->V;
    const cudaMemcpyKind in_kind = on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    float ms = 0.f;
    cudaError_t e = cudaMemcpyAsync(w->seeds, seed_vertices, sizeof(int) * kAdsL, cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w->pi, p_inj, sizeof(float) * V, in_kind, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(w->pc, p_cont, sizeof(float) * V, in_kind, g->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(w->mask, 0, sizeof(unsigned) * V, g->stream);
    if (e == cudaSuccess) {
        ads_seed_mask<<<1, 32, 0, g->stream>>>(w->seeds, kAdsL, w->mask);
        e = cudaGetLastError();
    }
    C2G_CUDA(e);
    if ((rc = ads_capture(g, w, iterations))) return rc;
    e = cudaEventRecord(g->ev0, g->stream);
    if (e == cudaSuccess) e = cudaGraphLaunch(w->exec, g->stream);
    if (e == cudaSuccess) e = cudaEventRecord(g->ev1, g->stream);
    if (e == cudaSuccess)
        e = cudaMemcpyAsync(Y_out, w->Y, sizeof(float) * V * kAdsL,
                            on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost, g->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, g->ev0, g->ev1);
    C2G_CUDA(e);
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->source = seed_vertices[0];
        stats->iterations = iterations;
        stats->edges_relaxed = (int64_t)g->E * iterations;
        stats->vertices_popped = (int64_t)g->V * iterations;
        stats->n_seeds = n_labels;
        stats->device_ms = ms;
        stats->alg_bytes = ((8.0 + 64.0) * (double)g->E + (64.0 + 64.0 + 12.0) * (double)g->V) * iterations;
    }
    return C2G_OK;
}
