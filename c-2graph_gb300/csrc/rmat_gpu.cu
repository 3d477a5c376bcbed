// R-MAT generation on the GPU: the same graph as the host writer (rmat.cpp), bit for bit.
//
// The host draws each edge's endpoints from a counter-based stream, drops self-loops,
// sorts every row and removes duplicates, then draws the weights per CSR index and
// normalises flist by the row's sum taken left to right in FP64.  Here: one thread per
// edge draw (rmat_draw.h, shared with the host), a radix sort of the (source, target)
// keys with the self-loops as the largest key, a unique pass, row bounds by binary
// search, and one thread per row for the weights, summing in the host's order.
#include <cub/cub.cuh>

#include <cmath>

#include "../../include/c2graph.h"
#include "host_io.h"
#include "internal.h"
#include "rmat.h"
#include "rmat_draw.h"

namespace c2g {

__global__ void rmat_edges_kernel(uint64_t seed, int scale, uint64_t ta, uint64_t tb, uint64_t tc, long long M,
                                  unsigned long long* keys) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < M; i += stride) {
        uint64_t s = 0, d = 0;
        rmat_endpoints(seed, (uint64_t)i, scale, ta, tb, tc, &s, &d);
        keys[i] = s == d ? ~0ull : (unsigned long long)((s << 32) | d);  // self-loops sort last
    }
}

// row[v] = index of the first key with source >= v (keys sorted, E of them).
__global__ void rmat_rows_kernel(const unsigned long long* __restrict__ keys, long long E, long long V, int* row) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v <= V; v += stride) {
        const unsigned long long k = (unsigned long long)v << 32;
        long long lo = 0, hi = E;
        while (lo < hi) {
            const long long mid = lo + ((hi - lo) >> 1);
            if (keys[mid] < k)
                lo = mid + 1;
            else
                hi = mid;
        }
        row[v] = (int)lo;
    }
}

__global__ void rmat_cols_kernel(const unsigned long long* __restrict__ keys, long long E, int* col) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < E; e += stride)
        col[e] = (int)(keys[e] & 0xffffffffull);
}

// One thread per row: the weights of its edges and flist normalised by the row's sum,
// accumulated left to right as the host does.
__global__ void rmat_weights_kernel(const int* __restrict__ row, long long V, uint64_t seed, int32_t wmin,
                                    uint64_t range, int* wgt, float* fw) {
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < V; v += stride) {
        const long long e0 = row[v], e1 = row[v + 1];
        double sum = 0.0;
        for (long long e = e0; e < e1; ++e) {
            wgt[e] = rmat_weight(seed, (uint64_t)e, wmin, range);
            const float u = rmat_fvalue(seed, (uint64_t)e);
            fw[e] = u;
            sum += (double)u;
        }
        for (long long e = e0; e < e1; ++e) fw[e] = (float)((double)fw[e] / sum);
    }
}

int rmat_build_gpu(int scale, int edge_factor, uint64_t seed, int32_t wmin, int32_t wmax, double a, double b,
                   double c, int device, RmatGraph& g) {
    if (scale < 1 || scale > 30 || edge_factor < 1)
        return fail(C2G_ERR_ARG, "rmat: bad scale %d / edge factor %d", scale, edge_factor);
    if (wmin > wmax) return fail(C2G_ERR_ARG, "rmat: wmin > wmax");
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0) return fail(C2G_ERR_ARG, "rmat: bad quadrant probabilities");
    const long long V = 1ll << scale;
    const long long M = (long long)edge_factor * V;
    if (M >= (1ll << 31)) return fail(C2G_ERR_ARG, "rmat: too many edges for int32 CSR");
    const double two32 = 4294967296.0;
    const uint64_t ta = (uint64_t)std::floor(a * two32);
    const uint64_t tb = ta + (uint64_t)std::floor(b * two32);
    const uint64_t tc = tb + (uint64_t)std::floor(c * two32);
    const uint64_t range = (uint64_t)((int64_t)wmax - (int64_t)wmin + 1);

    int prev = -1;
    cudaGetDevice(&prev);
    if (cudaSetDevice(device) != cudaSuccess) return fail(C2G_ERR_CUDA, "rmat: no device %d", device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = (sms > 0 ? sms : 1) * 8;
    unsigned long long *keys = nullptr, *sorted = nullptr;
    int *num = nullptr, *row = nullptr, *col = nullptr, *wgt = nullptr;
    float* fw = nullptr;
    void* temp = nullptr;
    cudaError_t e = cudaSuccess;
    auto step = [&](cudaError_t r) {
        if (e == cudaSuccess) e = r;
    };
    step(cudaMalloc(&keys, sizeof(unsigned long long) * (size_t)M));
    step(cudaMalloc(&sorted, sizeof(unsigned long long) * (size_t)M));
    step(cudaMalloc(&num, sizeof(int)));
    size_t tsort = 0, tuniq = 0;
    if (e == cudaSuccess) {
        step(cub::DeviceRadixSort::SortKeys(nullptr, tsort, keys, sorted, (int)M));
        step(cub::DeviceSelect::Unique(nullptr, tuniq, sorted, keys, num, (int)M));
        step(cudaMalloc(&temp, tsort > tuniq ? tsort : tuniq));
    }
    long long E = 0;
    if (e == cudaSuccess) {
        rmat_edges_kernel<<<blocks, 256>>>(seed, scale, ta, tb, tc, M, keys);
        step(cudaGetLastError());
        step(cub::DeviceRadixSort::SortKeys(temp, tsort, keys, sorted, (int)M));
        step(cub::DeviceSelect::Unique(temp, tuniq, sorted, keys, num, (int)M));  // distinct keys into `keys`
        int n = 0;
        step(cudaMemcpy(&n, num, sizeof(int), cudaMemcpyDeviceToHost));
        E = n;
        if (e == cudaSuccess && E > 0) {
            unsigned long long last = 0;
            step(cudaMemcpy(&last, keys + (E - 1), sizeof(last), cudaMemcpyDeviceToHost));
            if (last == ~0ull) --E;  // the self-loop marker
        }
    }
    step(cudaMalloc(&row, sizeof(int) * (size_t)(V + 1)));
    step(cudaMalloc(&col, sizeof(int) * (size_t)(E > 0 ? E : 1)));
    step(cudaMalloc(&wgt, sizeof(int) * (size_t)(E > 0 ? E : 1)));
    step(cudaMalloc(&fw, sizeof(float) * (size_t)(E > 0 ? E : 1)));
    if (e == cudaSuccess) {
        rmat_rows_kernel<<<blocks, 256>>>(keys, E, V, row);
        rmat_cols_kernel<<<blocks, 256>>>(keys, E, col);
        rmat_weights_kernel<<<blocks, 256>>>(row, V, seed, wmin, range, wgt, fw);
        step(cudaGetLastError());
        g.V = V;
        g.row.resize((size_t)V + 1);
        g.col.resize((size_t)E);
        g.wgt.resize((size_t)E);
        g.fw.resize((size_t)E);
        step(cudaMemcpy(g.row.data(), row, sizeof(int) * (size_t)(V + 1), cudaMemcpyDeviceToHost));
        if (E > 0) {
            step(cudaMemcpy(g.col.data(), col, sizeof(int) * (size_t)E, cudaMemcpyDeviceToHost));
            step(cudaMemcpy(g.wgt.data(), wgt, sizeof(int) * (size_t)E, cudaMemcpyDeviceToHost));
            step(cudaMemcpy(g.fw.data(), fw, sizeof(float) * (size_t)E, cudaMemcpyDeviceToHost));
        }
    }
    void* ptrs[] = {keys, sorted, num, row, col, wgt, fw, temp};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (prev >= 0) cudaSetDevice(prev);
    if (e != cudaSuccess) return fail(C2G_ERR_CUDA, "rmat on the device: %s", cudaGetErrorString(e));
    return C2G_OK;
}

}  // namespace c2g

extern "C" int c2g_rmat_write_gpu(const char* dir, int scale, int edge_factor, uint64_t seed, int32_t wmin,
                                  int32_t wmax, double a, double b, double c, int device) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "rmat: dir is NULL");
    c2g::RmatGraph g;
    int rc = c2g::rmat_build_gpu(scale, edge_factor, seed, wmin, wmax, a, b, c, device, g);
    if (rc) return rc;
    return c2g::write_origin(dir, g);
}
