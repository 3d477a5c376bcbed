// Seeded R-MAT generator writing the reference's origin/ binary layout
// (utils/convert2binary.cpp:98-129: vlist int32[V+1], elist int32[E], wlist int32[E],
// flist float32[E]).  Stands in for the reference's text converter on synthetic inputs.
//
// Determinism: every random draw is a counter-based splitmix64 output keyed by
// (seed, stream, index), so the graph does not depend on the thread count, and all
// arithmetic is integer except the flist normalisation (double sum in row order,
// compiled without FMA contraction), so x86 and Arm hosts write identical files.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/c2graph.h"
#include "host_io.h"
#include "rmat.h"
#include "rmat_draw.h"

namespace c2g {


// Generate an R-MAT graph in memory.
int rmat_build(int scale, int edge_factor, uint64_t seed, int32_t wmin, int32_t wmax, double a,
               double b, double c, RmatGraph& g) {
    if (scale < 1 || scale > 30 || edge_factor < 1)
        return fail(C2G_ERR_ARG, "rmat: bad scale %d / edge factor %d", scale, edge_factor);
    if (wmin > wmax) return fail(C2G_ERR_ARG, "rmat: wmin > wmax");
    if (a < 0 || b < 0 || c < 0 || a + b + c > 1.0)
        return fail(C2G_ERR_ARG, "rmat: bad quadrant probabilities");
    const int64_t V = int64_t(1) << scale;
    const int64_t M = (int64_t)edge_factor * V;
    if (M >= (int64_t(1) << 31)) return fail(C2G_ERR_ARG, "rmat: too many edges for int32 CSR");
    const double two32 = 4294967296.0;
    const uint64_t ta = (uint64_t)std::floor(a * two32);
    const uint64_t tb = ta + (uint64_t)std::floor(b * two32);
    const uint64_t tc = tb + (uint64_t)std::floor(c * two32);

    std::vector<int32_t> src(M), dst(M);
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < M; ++i) {
        uint64_t s = 0, d = 0;
        rmat_endpoints(seed, (uint64_t)i, scale, ta, tb, tc, &s, &d);
        src[i] = (int32_t)s;
        dst[i] = (int32_t)d;
    }

    // Bucket by source (counting sort), then sort + dedup each row; drop self-loops.
    std::vector<int64_t> cnt(V + 1, 0);
    for (int64_t i = 0; i < M; ++i)
        if (src[i] != dst[i]) cnt[src[i] + 1]++;
    for (int64_t v = 0; v < V; ++v) cnt[v + 1] += cnt[v];
    std::vector<int32_t> bucket(cnt[V]);
    {
        std::vector<int64_t> cur(cnt.begin(), cnt.end() - 1);
        for (int64_t i = 0; i < M; ++i)
            if (src[i] != dst[i]) bucket[cur[src[i]]++] = dst[i];
    }
    std::vector<int32_t>().swap(src);
    std::vector<int32_t>().swap(dst);
    std::vector<int32_t> deg(V, 0);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < V; ++v) {
        int32_t* b0 = bucket.data() + cnt[v];
        int32_t* b1 = bucket.data() + cnt[v + 1];
        std::sort(b0, b1);
        deg[v] = (int32_t)(std::unique(b0, b1) - b0);
    }
    g.V = V;
    g.row.assign(V + 1, 0);
    for (int64_t v = 0; v < V; ++v) g.row[v + 1] = g.row[v] + deg[v];
    const int64_t E = g.row[V];
    g.col.resize(E);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < V; ++v)
        std::memcpy(g.col.data() + g.row[v], bucket.data() + cnt[v], sizeof(int32_t) * deg[v]);
    std::vector<int32_t>().swap(bucket);

    g.wgt.resize(E);
    g.fw.resize(E);
    const uint64_t range = (uint64_t)((int64_t)wmax - (int64_t)wmin + 1);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int64_t v = 0; v < V; ++v) {
        double sum = 0.0;
        for (int64_t e = g.row[v]; e < g.row[v + 1]; ++e) {
            g.wgt[e] = rmat_weight(seed, (uint64_t)e, wmin, range);
            const float u = rmat_fvalue(seed, (uint64_t)e);
            g.fw[e] = u;
            sum += (double)u;
        }
        for (int64_t e = g.row[v]; e < g.row[v + 1]; ++e) g.fw[e] = (float)((double)g.fw[e] / sum);
    }
    return C2G_OK;
}

int write_origin(const std::string& dir, const RmatGraph& g) {
    int rc;
    if ((rc = make_dir(dir)) || (rc = make_dir(dir + "/origin")) || (rc = make_dir(dir + "/sssp")) ||
        (rc = make_dir(dir + "/ppr")))
        return rc;
    const std::string o = dir + "/origin/";
    if ((rc = write_array4(o + "vlist.bin", g.row.data(), g.row.size()))) return rc;
    if ((rc = write_array4(o + "elist.bin", g.col.data(), g.col.size()))) return rc;
    if ((rc = write_array4(o + "wlist.bin", g.wgt.data(), g.wgt.size()))) return rc;
    if ((rc = write_array4(o + "flist.bin", g.fw.data(), g.fw.size()))) return rc;
    return C2G_OK;
}

}  // namespace c2g

extern "C" int c2g_rmat_write(const char* dir, int scale, int edge_factor, uint64_t seed,
                              int32_t wmin, int32_t wmax, double a, double b, double c) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "rmat: dir is NULL");
    c2g::RmatGraph g;
    int rc = c2g::rmat_build(scale, edge_factor, seed, wmin, wmax, a, b, c, g);
    if (rc) return rc;
    return c2g::write_origin(dir, g);
}
