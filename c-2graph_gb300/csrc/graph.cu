// Device ingest of a CSR graph: the reference copies vlist/elist/wlist to separate
// device arrays through an extra host copy (src/sssp/purn/DeviceMemory.cuh:48-67,
// vec_to_arr by value).  Here the raw arrays go host->device once and a kernel
// interleaves (target, weight) into one 8-byte record per edge, so the traversal
// kernels read each edge with a single coalesced load.
#include "internal.h"

namespace c2g {

__global__ void interleave_kernel(const int* __restrict__ col, const int* __restrict__ w, int2* __restrict__ adj,
                                  long long E) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride)
        adj[e] = make_int2(__ldg(col + e), __ldg(w + e));
}

// Build adj[E] on the device from host arrays col[E] and w[E] (w holds int32 weights
// or float bits).  Uses two temporary device arrays.
int build_adj(c2g_graph* g, const int32_t* col, const int32_t* w, int2** out) {
    const size_t E = (size_t)g->E;
    int2* adj = nullptr;
    int *dcol = nullptr, *dw = nullptr;
    C2G_CUDA(cudaMalloc(&adj, sizeof(int2) * (E ? E : 1)));
    *out = adj;
    if (E == 0) return C2G_OK;
    C2G_CUDA(cudaMalloc(&dcol, sizeof(int) * E));
    cudaError_t e = cudaMalloc(&dw, sizeof(int) * E);
    if (e != cudaSuccess) {
        cudaFree(dcol);
        C2G_CUDA(e);
    }
    e = cudaMemcpyAsync(dcol, col, sizeof(int) * E, cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dw, w, sizeof(int) * E, cudaMemcpyHostToDevice, g->stream);
    if (e == cudaSuccess) {
        const int blocks = g->num_sms * 4;
        interleave_kernel<<<blocks, 256, 0, g->stream>>>(dcol, dw, adj, (long long)E);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    cudaFree(dcol);
    cudaFree(dw);
    C2G_CUDA(e);
    return C2G_OK;
}

// One chunk of the streaming ingest (c2g_graph_load): n edges starting at edge `base`,
// read from page-locked host memory mapped into the device's address space.  Writes the
// (target, weight) records of every weight kind present and checks each target against
// V (the flag records the first bad edge; the target is still stored, never used as an
// index here).
__global__ void interleave_chunk_kernel(const int* __restrict__ col, const int* __restrict__ w,
                                        const int* __restrict__ f, int2* __restrict__ adj_w, int2* __restrict__ adj_f,
                                        long long base, long long n, int V, long long* bad) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        const int c = col[i];
        if ((unsigned)c >= (unsigned)V) atomicMin(reinterpret_cast<unsigned long long*>(bad), (unsigned long long)(base + i));
        if (adj_w) adj_w[base + i] = make_int2(c, w[i]);
        if (adj_f) adj_f[base + i] = make_int2(c, f[i]);
    }
}

int launch_interleave_chunk(c2g_graph* g, const int* col, const int* w, const int* f, int2* adj_w, int2* adj_f,
                            long long base, long long n, long long* bad) {
    interleave_chunk_kernel<<<g->num_sms * 4, 256, 0, g->stream>>>(col, w, f, adj_w, adj_f, base, n, g->V, bad);
    C2G_CUDA(cudaGetLastError());
    return C2G_OK;
}

__global__ void set_weight_bits_kernel(int2* __restrict__ adj, const int* __restrict__ w, long long E) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x; e < E; e += stride) adj[e].y = w[e];
}

void adjoint_free(c2g_graph* g);

// Replace the float edge weights (flist order) of a graph in place; the reverse CSR
// built for the adjoint is dropped and rebuilt on next use.
int set_float_weights(c2g_graph* g, const float* w, int on_device) {
    if (!g->adj_f) return fail(C2G_ERR_UNSUPPORTED, "graph has no float weights to replace");
    const size_t E = (size_t)g->E;
    if (E == 0) return C2G_OK;
    const int* src = reinterpret_cast<const int*>(w);
    int* tmp = nullptr;
    if (!on_device) {
        C2G_CUDA(cudaMalloc(&tmp, sizeof(int) * E));
        cudaError_t e = cudaMemcpyAsync(tmp, w, sizeof(int) * E, cudaMemcpyHostToDevice, g->stream);
        if (e != cudaSuccess) {
            cudaFree(tmp);
            C2G_CUDA(e);
        }
        src = tmp;
    }
    set_weight_bits_kernel<<<g->num_sms * 4, 256, 0, g->stream>>>(g->adj_f, src, (long long)E);
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaStreamSynchronize(g->stream);
    if (tmp) cudaFree(tmp);
    C2G_CUDA(e);
    adjoint_free(g);
    return C2G_OK;
}

}  // namespace c2g
