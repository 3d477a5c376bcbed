// C ABI entry points (include/c2graph.h): graph loading, source rules, seed selection
// and result/statistics copy-out around the traversal launches.
#include <cuda_runtime.h>

#include <cstring>
#include <string>
#include <vector>

#include "../../include/c2graph.h"
#include "host_io.h"
#include "internal.h"

namespace c2g {

int build_adj(c2g_graph* g, const int32_t* col, const int32_t* w, int2** out);
int stream_graph(c2g_graph* g, const std::string& elist_path, const std::string* w_path, const std::string* f_path);
void adjoint_free(c2g_graph* g);

static const int kNoSidecar = -2;

static void graph_release(c2g_graph* g) {
    if (!g) return;
    int prev = 0;
    cudaGetDevice(&prev);
    cudaSetDevice(g->device);
    sssp_free(g);
    ppr_free(g);
    batch_free(g);
    ppr_batch_free(g);
    ads_free(g);
    if (!g->borrowed) adjoint_free(g);
    if (!g->borrowed) {
        void* ptrs[] = {g->row, g->adj_w, g->adj_f, g->hv, g->he, g->hw, g->rec_of_vertex};
        for (void* p : ptrs)
            if (p) cudaFree(p);
    }
    if (g->ev0) cudaEventDestroy(g->ev0);
    if (g->ev1) cudaEventDestroy(g->ev1);
    if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
    cudaSetDevice(prev);
    delete g;
}

// RAII guard that makes the graph's device current for the duration of a call.
struct DeviceScope {
    int prev = -1;
    explicit DeviceScope(int dev) {
        if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
        cudaSetDevice(dev);
    }
    ~DeviceScope() {
        if (prev >= 0) cudaSetDevice(prev);
    }
};

static int graph_new(int device, c2g_graph** out) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return fail(C2G_ERR_NODEVICE, "no CUDA device available");
    }
    if (device < 0 || device >= n) return fail(C2G_ERR_ARG, "device %d out of range [0,%d)", device, n);
    c2g_graph* g = new c2g_graph();
    g->device = device;
    cudaError_t e = cudaSetDevice(device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&g->num_sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) g->own_stream = true;
    if (e == cudaSuccess) e = cudaEventCreate(&g->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&g->ev1);
    if (e != cudaSuccess) {
        graph_release(g);
        return fail(C2G_ERR_CUDA, "graph init: %s", cudaGetErrorString(e));
    }
    *out = g;
    return C2G_OK;
}

static int graph_fill_rows(c2g_graph* g, const std::vector<int32_t>& vlist) {
    g->V = (int32_t)vlist.size() - 1;
    g->h_row = vlist;
    C2G_CUDA(cudaMalloc(&g->row, sizeof(int32_t) * vlist.size()));
    C2G_CUDA(cudaMemcpyAsync(g->row, vlist.data(), sizeof(int32_t) * vlist.size(), cudaMemcpyHostToDevice,
                             g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    return C2G_OK;
}

static int graph_fill(c2g_graph* g, const std::vector<int32_t>& vlist, const int32_t* elist, int64_t E,
                      const int32_t* wlist, const float* flist) {
    int rc;
    if ((rc = graph_fill_rows(g, vlist))) return rc;
    g->E = E;
    if (wlist && (rc = build_adj(g, elist, wlist, &g->adj_w))) return rc;
    if (flist && (rc = build_adj(g, elist, reinterpret_cast<const int32_t*>(flist), &g->adj_f))) return rc;
    return C2G_OK;
}

static int records_fill(c2g_graph* g, int32_t R, const int32_t* hv, const int32_t* he, const void* hw, bool hw_float,
                        const int32_t* rec_vertex) {
    if (R < 0 || !hv) return fail(C2G_ERR_ARG, "records: bad count or NULL hvlist");
    if (hv[0] != 0) return fail(C2G_ERR_FORMAT, "hvlist[0] = %d, expected 0", hv[0]);
    for (int32_t r = 0; r < R; ++r)
        if (hv[r + 1] < hv[r]) return fail(C2G_ERR_FORMAT, "hvlist not monotone at %d", r);
    const int64_t H = hv[R];
    if (H > 0 && (!he || !hw)) return fail(C2G_ERR_ARG, "records: NULL helist/hwlist");
    for (int64_t k = 0; k < H; ++k)
        if (he[k] < 0 || he[k] >= g->V)
            return fail(C2G_ERR_FORMAT, "helist[%lld] = %d out of range", (long long)k, he[k]);
    for (void* p : {(void*)g->hv, (void*)g->he, (void*)g->hw, (void*)g->rec_of_vertex})
        if (p) cudaFree(p);
    g->hv = g->he = g->hw = g->rec_of_vertex = nullptr;
    g->R = R;
    g->H = H;
    g->hw_float = hw_float;
    g->h_hv.assign(hv, hv + R + 1);
    g->h_he.assign(he, he + H);
    g->h_hw.assign(reinterpret_cast<const int32_t*>(hw), reinterpret_cast<const int32_t*>(hw) + H);
    C2G_CUDA(cudaMalloc(&g->hv, sizeof(int32_t) * (R + 1)));
    C2G_CUDA(cudaMemcpyAsync(g->hv, hv, sizeof(int32_t) * (R + 1), cudaMemcpyHostToDevice, g->stream));
    C2G_CUDA(cudaMalloc(&g->he, sizeof(int32_t) * (H ? H : 1)));
    C2G_CUDA(cudaMalloc(&g->hw, sizeof(int32_t) * (H ? H : 1)));
    if (H) {
        C2G_CUDA(cudaMemcpyAsync(g->he, he, sizeof(int32_t) * H, cudaMemcpyHostToDevice, g->stream));
        C2G_CUDA(cudaMemcpyAsync(g->hw, hw, sizeof(int32_t) * H, cudaMemcpyHostToDevice, g->stream));
    }
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    g->h_rec_of_vertex.clear();
    if (rec_vertex) {
        g->h_rec_of_vertex.assign((size_t)g->V, -1);
        for (int32_t r = 0; r < R; ++r) {
            const int32_t v = rec_vertex[r];
            if (v < 0 || v >= g->V) return fail(C2G_ERR_FORMAT, "hvmap[%d] = %d out of range", r, v);
            g->h_rec_of_vertex[v] = r;
        }
    }
    return C2G_OK;
}

static int stats_fill(c2g_graph* g, const TraversalCtl* dctl, int32_t source, float ms, bool ppr, c2g_stats* st) {
    TraversalCtl ctl;
    C2G_CUDA(cudaMemcpyAsync(&ctl, dctl, sizeof(ctl), cudaMemcpyDeviceToHost, g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    std::memcpy(g->last_phase_ns, ctl.phase_ns, sizeof(g->last_phase_ns));
    if (ctl.flags & (C2G_FLAG_BARRIER_TIMEOUT | C2G_FLAG_QUEUE_OVERFLOW | C2G_FLAG_BOUNDS)) {
        // The launch ended early: force the stamp arrays to be reset by the next launch.
        static const StampState reset{1 << 30, 1 << 30, {0, 0}};
        StampState* dst = ppr ? g->ppr.st : g->sssp.st;
        cudaMemcpyAsync(dst, &reset, sizeof(reset), cudaMemcpyHostToDevice, g->stream);
        cudaStreamSynchronize(g->stream);
    }
    if (st) {
        std::memset(st, 0, sizeof(*st));
        st->source = source;
        st->iterations = ctl.iterations;
        st->vertices_popped = ctl.popped;
        st->edges_relaxed = ctl.relaxed;
        st->touched = ctl.touched;
        st->n_seeds = ctl.seeds;
        st->device_ms = ms;
        st->status_flags = ctl.flags;
        const double V = (double)g->V;
        // Byte model: SSSP 4V + 16 per popped vertex + 12 per relaxed edge;
        // push 12V + 20 per popped vertex + 12 per pushed edge.
        st->alg_bytes = ppr ? 12.0 * V + 20.0 * (double)ctl.popped + 12.0 * (double)ctl.relaxed
                            : 4.0 * V + 16.0 * (double)ctl.popped + 12.0 * (double)ctl.relaxed;
    }
    if (ctl.flags & C2G_FLAG_BARRIER_TIMEOUT) return fail(C2G_ERR_TIMEOUT, "grid barrier wait ran out");
    if (ctl.flags & C2G_FLAG_QUEUE_OVERFLOW) return fail(C2G_ERR_OVERFLOW, "frontier queue overflow");
    if (ctl.flags & C2G_FLAG_BOUNDS) return fail(C2G_ERR_OVERFLOW, "device index check failed");
    return C2G_OK;
}

static bool is_device_ptr(const void* p) {
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// Seeds of `source` in the record arrays under `mode`; n = -1 when unavailable.
static int record_range(const c2g_graph* g, int32_t source, int mode, int32_t* first, int32_t* n) {
    *first = 0;
    *n = 0;
    if (g->R < 0) return fail(C2G_ERR_UNSUPPORTED, "graph has no pruned records (hvlist)");
    int32_t r;
    if (mode == C2G_SEEDS_COMPAT) {
        // The reference reads hvlist[source] and hvlist[source+1]; beyond the record count
        // that read is out of bounds, reported here as a range error.
        if (source + 1 > g->R)
            return fail(C2G_ERR_RANGE, "COMPAT seeds: source %d >= record count %d", source, g->R);
        r = source;
    } else if (mode == C2G_SEEDS_EXACT) {
        if (g->h_rec_of_vertex.empty())
            return fail(C2G_ERR_UNSUPPORTED, "EXACT seeds need the record->vertex sidecar (hvmap.bin)");
        r = g->h_rec_of_vertex[source];
        if (r < 0) return C2G_OK;
    } else {
        return fail(C2G_ERR_ARG, "bad seed mode %d", mode);
    }
    *first = g->h_hv[r];
    *n = g->h_hv[r + 1] - g->h_hv[r];
    return C2G_OK;
}

int graph_view(c2g_graph* base, c2g_graph** out) {
    c2g_graph* g = nullptr;
    int rc = graph_new(base->device, &g);
    if (rc) return rc;
    g->variant = base->variant;
    g->V = base->V;
    g->E = base->E;
    g->row = base->row;
    g->adj_w = base->adj_w;
    g->adj_f = base->adj_f;
    g->row_r = base->row_r;
    g->adj_r = base->adj_r;
    g->adj_rw = base->adj_rw;
    g->mark_r = base->mark_r;
    g->mark_f = base->mark_f;
    g->R = base->R;
    g->H = base->H;
    g->hv = base->hv;
    g->he = base->he;
    g->hw = base->hw;
    g->hw_float = base->hw_float;
    g->rec_of_vertex = base->rec_of_vertex;
    g->h_row = base->h_row;
    g->h_hv = base->h_hv;
    g->h_rec_of_vertex = base->h_rec_of_vertex;
    g->h_he = base->h_he;
    g->h_hw = base->h_hw;
    g->sssp_cfg = base->sssp_cfg;
    g->ppr_cfg = base->ppr_cfg;
    g->wstat_valid = base->wstat_valid;
    g->wstat_wmax_bits = base->wstat_wmax_bits;
    g->borrowed = true;
    *out = g;
    return C2G_OK;
}

void graph_free_view(c2g_graph* g) { graph_release(g); }

}  // namespace c2g

using namespace c2g;

extern "C" {

int c2g_abi_version(void) { return C2G_ABI_VERSION; }
const char* c2g_last_error(void) { return c2g::last_error(); }

int c2g_device_count(int* count) {
    if (!count) return fail(C2G_ERR_ARG, "count is NULL");
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        n = 0;
    }
    *count = n;
    return C2G_OK;
}

int c2g_graph_create(int device, int32_t V, int64_t E, const int32_t* vlist, const int32_t* elist,
                     const int32_t* wlist, const float* flist, c2g_graph** out) {
    if (!out || !vlist || (E > 0 && !elist)) return fail(C2G_ERR_ARG, "graph_create: NULL argument");
    if (V < 0 || E < 0 || E >= (int64_t(1) << 31)) return fail(C2G_ERR_ARG, "graph_create: bad sizes");
    if (!wlist && !flist) return fail(C2G_ERR_ARG, "graph_create: need wlist or flist");
    *out = nullptr;
    std::vector<int32_t> vl(vlist, vlist + V + 1);
    std::vector<int32_t> el(elist, elist + E);
    int rc = check_csr(vl, el);
    if (rc) return rc;
    c2g_graph* g = nullptr;
    if ((rc = graph_new(device, &g))) return rc;
    DeviceScope ds(device);
    if ((rc = graph_fill(g, vl, elist, E, wlist, flist))) {
        graph_release(g);
        return rc;
    }
    g->variant = C2G_GRAPH_ORIGIN;
    *out = g;
    return C2G_OK;
}

int c2g_graph_load(const char* dir, int variant, int device, c2g_graph** out) {
    if (!dir || !out) return fail(C2G_ERR_ARG, "graph_load: NULL argument");
    *out = nullptr;
    const std::string base(dir);
    std::string sub;
    switch (variant) {
        case C2G_GRAPH_ORIGIN: sub = "/origin/"; break;
        case C2G_GRAPH_SSSP: sub = "/sssp/"; break;
        case C2G_GRAPH_PPR: sub = "/ppr/"; break;
        default: return fail(C2G_ERR_ARG, "bad graph variant %d", variant);
    }
    const std::string d = base + sub;
    std::vector<int32_t> vlist, hv, he, hwi, hvmap;
    std::vector<float> hwf;
    int rc;
    if ((rc = read_array4(d + "vlist.bin", vlist))) return rc;
    // Edge arrays are streamed from their files (stream_load.cpp); which weight kinds:
    std::string wpath, fpath;
    if (variant == C2G_GRAPH_ORIGIN) {
        if (file_exists(d + "wlist.bin")) wpath = d + "wlist.bin";
        if (file_exists(d + "flist.bin")) fpath = d + "flist.bin";
        if (wpath.empty() && fpath.empty()) return fail(C2G_ERR_IO, "file:%swlist.bin not exist.", d.c_str());
    } else if (variant == C2G_GRAPH_SSSP) {
        wpath = d + "wlist.bin";
    } else {
        fpath = d + "wlist.bin";  // ppr/wlist.bin holds float weights
    }
    if (!file_exists(d + "elist.bin")) return fail(C2G_ERR_IO, "file:%selist.bin not exist.", d.c_str());
    for (const std::string* path : {&wpath, &fpath})
        if (!path->empty() && !file_exists(*path)) return fail(C2G_ERR_IO, "file:%s not exist.", path->c_str());
    if (variant == C2G_GRAPH_SSSP) {
        if ((rc = read_array4(d + "hvlist.bin", hv))) return rc;
        if ((rc = read_array4(d + "helist.bin", he))) return rc;
        if ((rc = read_array4(d + "hwlist.bin", hwi))) return rc;
        if (file_exists(d + "hvmap.bin") && (rc = read_array4(d + "hvmap.bin", hvmap))) return rc;
    } else if (variant == C2G_GRAPH_PPR) {
        if ((rc = read_array4(d + "hvlist.bin", hv))) return rc;
        if ((rc = read_array4(d + "helist.bin", he))) return rc;
        if ((rc = read_array4(d + "hwlist.bin", hwf))) return rc;
    }
    if ((rc = check_rows(vlist))) return rc;
    if (variant != C2G_GRAPH_ORIGIN) {
        if (hv.empty()) return fail(C2G_ERR_FORMAT, "%shvlist.bin is empty", d.c_str());
        const int64_t H = hv.back();
        const size_t hwn = variant == C2G_GRAPH_SSSP ? hwi.size() : hwf.size();
        if (H < 0 || (int64_t)he.size() < H || (int64_t)hwn < H)
            return fail(C2G_ERR_FORMAT, "record arrays shorter than hvlist[R] = %lld", (long long)H);
        if (!hvmap.empty() && hvmap.size() != hv.size() - 1)
            return fail(C2G_ERR_FORMAT, "hvmap.bin has %zu entries for %zu records", hvmap.size(), hv.size() - 1);
    }
    c2g_graph* g = nullptr;
    if ((rc = graph_new(device, &g))) return rc;
    DeviceScope ds(device);
    if ((rc = graph_fill_rows(g, vlist)) ||
        (rc = stream_graph(g, d + "elist.bin", wpath.empty() ? nullptr : &wpath, fpath.empty() ? nullptr : &fpath))) {
        graph_release(g);
        return rc;
    }
    g->variant = variant;
    if (variant != C2G_GRAPH_ORIGIN) {
        const void* hw = variant == C2G_GRAPH_SSSP ? (const void*)hwi.data() : (const void*)hwf.data();
        rc = records_fill(g, (int32_t)hv.size() - 1, hv.data(), he.data(), hw, variant == C2G_GRAPH_PPR,
                          hvmap.empty() ? nullptr : hvmap.data());
        if (rc) {
            graph_release(g);
            return rc;
        }
    }
    *out = g;
    return C2G_OK;
}

int c2g_graph_set_records(c2g_graph* g, int32_t R, const int32_t* hvlist, const int32_t* helist,
                          const void* hwlist, int hw_is_float, const int32_t* record_vertex) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    std::lock_guard<std::mutex> lk(g->mu);
    DeviceScope ds(g->device);
    return records_fill(g, R, hvlist, helist, hwlist, hw_is_float != 0, record_vertex);
}

void c2g_graph_free(c2g_graph* g) { graph_release(g); }

int c2g_graph_info(const c2g_graph* g, int32_t* V, int64_t* E, int32_t* R) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    if (V) *V = g->V;
    if (E) *E = g->E;
    if (R) *R = g->R;
    return C2G_OK;
}

int c2g_graph_set_stream(c2g_graph* g, void* stream) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    std::lock_guard<std::mutex> lk(g->mu);
    DeviceScope ds(g->device);
    // Work already queued on the old stream (workspace initialisation included) must
    // finish before the new stream takes over.
    if (g->stream) C2G_CUDA(cudaStreamSynchronize(g->stream));
    if (g->own_stream && g->stream) cudaStreamDestroy(g->stream);
    g->own_stream = false;
    g->stream = (cudaStream_t)stream;
    return C2G_OK;
}

int c2g_sssp_set_config(c2g_graph* g, int32_t delta, int32_t tile, int32_t max_iter) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    int lt = 0;
    while ((1 << lt) < tile) ++lt;
    if (tile < 32 || tile > 4096 || (1 << lt) != tile) return fail(C2G_ERR_ARG, "tile %d not a power of two in [32,4096]", tile);
    if (max_iter < 1) return fail(C2G_ERR_ARG, "max_iter must be >= 1");
    std::lock_guard<std::mutex> lk(g->mu);
    g->sssp_cfg.delta = delta > 0 ? delta : 0;
    g->sssp_cfg.log_tile = lt;
    g->sssp_cfg.max_iter = max_iter;
    return C2G_OK;
}

int c2g_graph_last_phases(const c2g_graph* g, double ms[4]) {
    if (!g || !ms) return fail(C2G_ERR_ARG, "NULL argument");
    for (int k = 0; k < 4; ++k) ms[k] = (double)g->last_phase_ns[k] * 1e-6;
    return C2G_OK;
}

int c2g_graph_last_rounds(c2g_graph* g, int32_t cap, double* ms, double* first_ms, int64_t* work, int32_t* shape,
                          int32_t* n) {
    if (!g || !n) return fail(C2G_ERR_ARG, "NULL argument");
    *n = 0;
    std::lock_guard<std::mutex> lk(g->mu);
    if (!g->last_trace) return C2G_OK;
    DeviceScope ds(g->device);
    std::vector<RoundTrace> t((size_t)kMaxTraceRounds + 1);
    C2G_CUDA(cudaMemcpyAsync(t.data(), g->last_trace, sizeof(RoundTrace) * t.size(), cudaMemcpyDeviceToHost,
                             g->stream));
    C2G_CUDA(cudaStreamSynchronize(g->stream));
    int rounds = -1;
    for (int i = 0; i <= kMaxTraceRounds; ++i)
        if (t[(size_t)i].shape == -1) {
            rounds = i;
            break;
        }
    if (rounds < 0) return C2G_OK;  // the launch did not finish cleanly: no trace
    for (int i = 0; i < rounds && i < cap; ++i) {
        if (ms) ms[i] = (double)(t[(size_t)i + 1].t_ns - t[(size_t)i].t_ns) * 1e-6;
        if (first_ms) first_ms[i] = (double)t[(size_t)i].mid_ns * 1e-6;
        if (work) work[i] = t[(size_t)i].work;
        if (shape) shape[i] = t[(size_t)i].shape;
    }
    *n = rounds;
    return C2G_OK;
}

int c2g_graph_set_watchdog(c2g_graph* g, int32_t barrier_timeout_ms, int32_t stall_next_sssp) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    if (barrier_timeout_ms < 0) return fail(C2G_ERR_ARG, "barrier_timeout_ms must be >= 0");
    std::lock_guard<std::mutex> lk(g->mu);
    g->barrier_ns = (unsigned long long)barrier_timeout_ms * 1000000ull;
    g->stall_next_sssp = stall_next_sssp ? 1 : 0;
    return C2G_OK;
}

int c2g_ppr_set_config(c2g_graph* g, int32_t pull_div, int32_t dense_div) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    if (pull_div < 0 || dense_div < 0) return fail(C2G_ERR_ARG, "pull_div and dense_div must be >= 0");
    std::lock_guard<std::mutex> lk(g->mu);
    g->ppr_cfg.pull_div = pull_div;
    g->ppr_cfg.dense_div = dense_div;
    return C2G_OK;
}

int c2g_ppr_batch_set_pull(c2g_graph* g, float ratio) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    if (ratio != ratio) return fail(C2G_ERR_ARG, "ratio is NaN");
    std::lock_guard<std::mutex> lk(g->mu);
    g->ppr_cfg.batch_pull_ratio = ratio;
    return C2G_OK;
}

int c2g_sssp_batch_set_pull(c2g_graph* g, float frac) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    if (frac != frac) return fail(C2G_ERR_ARG, "frac is NaN");
    std::lock_guard<std::mutex> lk(g->mu);
    g->sssp_cfg.batch_pull_frac = frac;
    return C2G_OK;
}

int c2g_sssp_batch_get_pull(const c2g_graph* g, float* frac) {
    if (!g || !frac) return fail(C2G_ERR_ARG, "NULL argument");
    *frac = g->sssp_cfg.batch_pull_frac;
    return C2G_OK;
}

static int log2_exact(int32_t x) {
    int l = 0;
    while (l < 31 && (1 << l) < x) ++l;
    return (1 << l) == x ? l : -1;
}

int c2g_sssp_batch_set_tile(c2g_graph* g, int32_t big_steps, int32_t min_tiles_per_warp) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    const int lb = log2_exact(big_steps), lm = log2_exact(min_tiles_per_warp);
    if (lb < 7 || lb > 12) return fail(C2G_ERR_ARG, "big_steps must be a power of two in [128, 4096]");
    if (lm < 0 || lm > 10) return fail(C2G_ERR_ARG, "min_tiles_per_warp must be a power of two in [1, 1024]");
    std::lock_guard<std::mutex> lk(g->mu);
    g->sssp_cfg.batch_tile_big_log = lb;
    g->sssp_cfg.batch_tile_min_log = lm;
    return C2G_OK;
}

int c2g_sssp_batch_get_tile(const c2g_graph* g, int32_t* big_steps, int32_t* min_tiles_per_warp) {
    if (!g) return fail(C2G_ERR_ARG, "graph is NULL");
    if (big_steps) *big_steps = 1 << g->sssp_cfg.batch_tile_big_log;
    if (min_tiles_per_warp) *min_tiles_per_warp = 1 << g->sssp_cfg.batch_tile_min_log;
    return C2G_OK;
}

int c2g_sssp_resolve_source(const c2g_graph* g, int32_t source, int pruned, int mode, int32_t* adjusted) {
    if (!g || !adjusted) return fail(C2G_ERR_ARG, "NULL argument");
    for (int32_t s = source;; ++s) {
        if (s < 0 || s >= g->V) return fail(C2G_ERR_RANGE, "no eligible source at or after %d (V = %d)", source, g->V);
        if (g->h_row[s + 1] - g->h_row[s] < 1) continue;
        if (pruned) {
            int32_t first, n;
            int rc = record_range(g, s, mode, &first, &n);
            if (rc) return rc;
            if (n > 1000) continue;
        }
        *adjusted = s;
        return C2G_OK;
    }
}

int c2g_sssp(c2g_graph* g, int32_t source, int use_seeds, int seed_mode, int32_t* dist, int dist_on_device,
             c2g_stats* stats) {
    if (!g || !dist) return fail(C2G_ERR_ARG, "NULL argument");
    if (source < 0 || source >= g->V) return fail(C2G_ERR_RANGE, "source %d out of range [0,%d)", source, g->V);
    std::lock_guard<std::mutex> lk(g->mu);
    DeviceScope ds(g->device);
    int32_t first = 0, n = 0;
    int rc;
    if (use_seeds && (rc = record_range(g, source, seed_mode, &first, &n))) return rc;
    if (dist_on_device && !is_device_ptr(dist)) return fail(C2G_ERR_ARG, "dist is not a device pointer");
    float ms = 0.f;
    rc = sssp_launch(g, source, n ? g->he + first : nullptr, n ? g->hw + first : nullptr, n,
                     dist_on_device ? dist : nullptr, &ms);
    if (rc) return rc;
    if (!dist_on_device)
        C2G_CUDA(cudaMemcpyAsync(dist, g->sssp.dist, sizeof(int32_t) * (size_t)g->V, cudaMemcpyDeviceToHost, g->stream));
    return stats_fill(g, g->sssp.ctl, source, ms, false, stats);
}

int c2g_sssp_batch(c2g_graph* g, int32_t n, const int32_t* sources, int use_seeds, int seed_mode, int32_t* dist,
                   int dist_on_device, int layout, c2g_stats* stats) {
    if (!g || !sources || !dist) return fail(C2G_ERR_ARG, "NULL argument");
    if (n < 1) return fail(C2G_ERR_ARG, "batch needs at least one source");
    if (layout != C2G_LAYOUT_QUERY_MAJOR && layout != C2G_LAYOUT_VERTEX_MAJOR)
        return fail(C2G_ERR_ARG, "bad layout %d", layout);
    for (int32_t i = 0; i < n; ++i)
        if (sources[i] < 0 || sources[i] >= g->V)
            return fail(C2G_ERR_RANGE, "source %d (entry %d) out of range [0,%d)", sources[i], i, g->V);
    std::lock_guard<std::mutex> lk(g->mu);
    DeviceScope ds(g->device);
    std::vector<int32_t> off, sv, sw;
    if (use_seeds) {
        off.reserve((size_t)n + 1);
        off.push_back(0);
        for (int32_t i = 0; i < n; ++i) {
            int32_t first = 0, cnt = 0;
            int rc = record_range(g, sources[i], seed_mode, &first, &cnt);
            if (rc) return rc;
            sv.insert(sv.end(), g->h_he.begin() + first, g->h_he.begin() + first + cnt);
            sw.insert(sw.end(), g->h_hw.begin() + first, g->h_hw.begin() + first + cnt);
            off.push_back((int32_t)sv.size());
        }
    }
    if (dist_on_device && !is_device_ptr(dist)) return fail(C2G_ERR_ARG, "dist is not a device pointer");
    float ms = 0.f;
    long long counters[2] = {0, 0};
    TraversalCtl ctl;
    int rc = sssp_batch_launch(g, n, sources, use_seeds ? &off : nullptr, use_seeds ? &sv : nullptr,
                               use_seeds ? &sw : nullptr, dist, dist_on_device, layout == C2G_LAYOUT_QUERY_MAJOR, &ms,
                               counters, &ctl);
    if (rc) return rc;
    std::memcpy(g->last_phase_ns, ctl.phase_ns, sizeof(g->last_phase_ns));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->source = sources[0];
        stats->iterations = ctl.iterations;
        stats->vertices_popped = ctl.popped;  // (vertex, 32-query word) entries
        stats->edges_relaxed = counters[0];   // (query, edge) relaxations
        stats->touched = ctl.relaxed;         // edge x word steps
        stats->n_seeds = (int64_t)sv.size();
        stats->device_ms = ms;
        stats->status_flags = ctl.flags;
        // Byte model: 40 per entry (id + bounds + 32 B mask word/row share) + 8 per
        // edge-word step + 8 per (query, edge) relaxation (4 B read + 4 B atomic), plus
        // the 4 B x V x Q initialisation.
        stats->alg_bytes = 40.0 * (double)ctl.popped + 8.0 * (double)ctl.relaxed + 8.0 * (double)counters[0] +
                           4.0 * (double)g->V * (double)((n + 31) / 32 * 32);
    }
    if (ctl.flags & C2G_FLAG_BARRIER_TIMEOUT) return fail(C2G_ERR_TIMEOUT, "grid barrier wait ran out");
    if (ctl.flags & C2G_FLAG_QUEUE_OVERFLOW) return fail(C2G_ERR_OVERFLOW, "frontier queue overflow");
    if (ctl.flags & C2G_FLAG_BOUNDS) return fail(C2G_ERR_OVERFLOW, "device index check failed");
    return C2G_OK;
}

int c2g_ppr_batch(c2g_graph* g, int32_t n, const int32_t* sources, const c2g_ppr_params* params, float* pr,
                  float* res, int on_device, int layout, c2g_stats* stats) {
    if (!g || !sources || !params || !pr) return fail(C2G_ERR_ARG, "NULL argument");
    if (n < 1) return fail(C2G_ERR_ARG, "batch needs at least one source");
    if (layout != C2G_LAYOUT_QUERY_MAJOR && layout != C2G_LAYOUT_VERTEX_MAJOR)
        return fail(C2G_ERR_ARG, "bad layout %d", layout);
    if (!(params->alpha > 0.f && params->alpha <= 1.f)) return fail(C2G_ERR_ARG, "alpha must be in (0,1]");
    if (!(params->rmax >= 0.f)) return fail(C2G_ERR_ARG, "rmax must be >= 0");
    if (params->max_iter < 1) return fail(C2G_ERR_ARG, "max_iter must be >= 1");
    for (int32_t i = 0; i < n; ++i)
        if (sources[i] < 0 || sources[i] >= g->V)
            return fail(C2G_ERR_RANGE, "source %d (entry %d) out of range [0,%d)", sources[i], i, g->V);
    std::lock_guard<std::mutex> lk(g->mu);
    DeviceScope ds(g->device);
    std::vector<int32_t> off, sv;
    std::vector<float> sw;
    if (params->seeded) {
        if (g->R < 0 || !g->hw_float) return fail(C2G_ERR_UNSUPPORTED, "seeded push needs ppr/ records");
        if (g->R != g->V) return fail(C2G_ERR_FORMAT, "ppr/ hvlist has %d records for %d vertices", g->R, g->V);
        off.push_back(0);
        for (int32_t i = 0; i < n; ++i) {
            const int32_t s = sources[i], first = g->h_hv[s], cnt = g->h_hv[s + 1] - first;
            sv.insert(sv.end(), g->h_he.begin() + first, g->h_he.begin() + first + cnt);
            for (int32_t k = 0; k < cnt; ++k) {
                float f;
                std::memcpy(&f, &g->h_hw[first + k], sizeof(f));
                sw.push_back(f);
            }
            off.push_back((int32_t)sv.size());
        }
    }
    if (on_device && (!is_device_ptr(pr) || (res && !is_device_ptr(res))))
        return fail(C2G_ERR_ARG, "pr/res are not device pointers");
    float ms = 0.f;
    long long counters[2] = {0, 0};
    TraversalCtl ctl;
    int rc = ppr_batch_launch(g, n, sources, *params, params->seeded ? &off : nullptr, params->seeded ? &sv : nullptr,
                              params->seeded ? &sw : nullptr, pr, res, on_device, layout == C2G_LAYOUT_QUERY_MAJOR,
                              &ms, counters, &ctl);
    if (rc) return rc;
    std::memcpy(g->last_phase_ns, ctl.phase_ns, sizeof(g->last_phase_ns));
    if (stats) {
        std::memset(stats, 0, sizeof(*stats));
        stats->source = sources[0];
        stats->iterations = ctl.iterations;
        stats->vertices_popped = ctl.popped;
        stats->edges_relaxed = counters[0];
        stats->touched = ctl.touched;
        stats->n_seeds = (int64_t)sv.size();
        stats->device_ms = ms;
        stats->status_flags = ctl.flags;
        // 40 per frontier entry + 8 per edge-word step + 8 per (query, edge) push (FP64
        // message add) + 32 per touched (vertex, query) lane (res and msg read and
        // write) + the pr/res initialisation (12 per vertex and query).
        const double Qp = (double)((n + 31) / 32 * 32);
        stats->alg_bytes = 40.0 * (double)ctl.popped + 8.0 * (double)ctl.relaxed + 8.0 * (double)counters[0] +
                           32.0 * (double)ctl.touched + 12.0 * (double)g->V * Qp;
    }
    if (ctl.flags & C2G_FLAG_BARRIER_TIMEOUT) return fail(C2G_ERR_TIMEOUT, "grid barrier wait ran out");
    if (ctl.flags & C2G_FLAG_QUEUE_OVERFLOW) return fail(C2G_ERR_OVERFLOW, "frontier queue overflow");
    if (ctl.flags & C2G_FLAG_BOUNDS) return fail(C2G_ERR_OVERFLOW, "device index check failed");
    return C2G_OK;
}

int c2g_ppr_default_params(const c2g_graph* g, int adsorption, c2g_ppr_params* out) {
    if (!g || !out) return fail(C2G_ERR_ARG, "NULL argument");
    if (!adsorption) {
        out->alpha = 0.2f;                                  // src/ppr/purn/Main.cu:66
        out->rmax = 0.001f / (float)((int64_t)g->V + 1);    // :67
        out->r0 = 1.0f;
        out->pr0 = 0.2f;
        out->max_iter = 500;                                // :224
        out->seeded = g->variant == C2G_GRAPH_PPR ? 1 : 0;
    } else {
        out->alpha = 0.2f;                                  // src/adsorption/w-base/Main.cu:63
        out->rmax = 1.0f / (float)(g->V > 0 ? g->V : 1);    // :64
        out->r0 = 10.0f;                                    // :149
        out->pr0 = 8.0f;                                    // :152, 0.8 * 10
        out->max_iter = 2000;                               // :186
        out->seeded = 0;
    }
    return C2G_OK;
}

int c2g_ppr(c2g_graph* g, int32_t source, const c2g_ppr_params* params, float* pr, float* res, int on_device,
            c2g_stats* stats) {
    if (!g || !params || !pr) return fail(C2G_ERR_ARG, "NULL argument");
    if (source < 0 || source >= g->V) return fail(C2G_ERR_RANGE, "source %d out of range [0,%d)", source, g->V);
    if (!(params->alpha > 0.f && params->alpha <= 1.f)) return fail(C2G_ERR_ARG, "alpha must be in (0,1]");
    if (!(params->rmax >= 0.f)) return fail(C2G_ERR_ARG, "rmax must be >= 0");
    if (params->max_iter < 1) return fail(C2G_ERR_ARG, "max_iter must be >= 1");
    std::lock_guard<std::mutex> lk(g->mu);
    DeviceScope ds(g->device);
    int32_t first = 0, n = 0;
    if (params->seeded) {
        if (g->R < 0 || !g->hw_float) return fail(C2G_ERR_UNSUPPORTED, "seeded push needs ppr/ records");
        if (g->R != g->V) return fail(C2G_ERR_FORMAT, "ppr/ hvlist has %d records for %d vertices", g->R, g->V);
        first = g->h_hv[source];
        n = g->h_hv[source + 1] - first;
    }
    if (on_device && (!is_device_ptr(pr) || (res && !is_device_ptr(res))))
        return fail(C2G_ERR_ARG, "pr/res are not device pointers");
    float ms = 0.f;
    int rc = ppr_launch(g, source, *params, n ? g->he + first : nullptr,
                        n ? reinterpret_cast<const float*>(g->hw + first) : nullptr, n, on_device ? pr : nullptr,
                        on_device ? res : nullptr, &ms);
    if (rc) return rc;
    if (!on_device) {
        C2G_CUDA(cudaMemcpyAsync(pr, g->ppr.pr, sizeof(float) * (size_t)g->V, cudaMemcpyDeviceToHost, g->stream));
        if (res)
            C2G_CUDA(cudaMemcpyAsync(res, g->ppr.res_f, sizeof(float) * (size_t)g->V, cudaMemcpyDeviceToHost, g->stream));
    }
    return stats_fill(g, g->ppr.ctl, source, ms, true, stats);
}

}  // extern "C"
