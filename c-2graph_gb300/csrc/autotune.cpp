// Autotuner of the SSSP kernel's tile and bucket (near/far delta) parameters.
//
// The reference hard-codes its launch geometry (core/Util.cuh:31-34) and has no bucket
// parameter.  Here the best (delta, tile) depends on the graph's weight range and degree
// skew, so c2g_sssp_autotune times every candidate on sample sources.  A candidate whose
// distances differ from the first candidate's is rejected (all must be the same
// fixed point).  The winner is applied to the handle and, when a path is given, written
// as a JSON record of every timing.
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/c2graph.h"
#include "host_io.h"
#include "internal.h"

extern "C" int c2g_sssp_autotune(c2g_graph* g, int32_t n, const int32_t* sources, int use_seeds, int seed_mode,
                                 const char* json_path, int32_t* best_delta, int32_t* best_tile) {
    using namespace c2g;
    if (!g || !sources || n < 1) return fail(C2G_ERR_ARG, "autotune: need sample sources");
    const int deltas[] = {0, 50, 100, 200, 400, 800, 1600, 3200};
    const int tiles[] = {64, 128, 256, 512, 1024};
    const int32_t V = g->V;
    std::vector<std::vector<int32_t>> ref(n, std::vector<int32_t>((size_t)V));
    std::vector<int32_t> dist((size_t)V);
    const SsspConfig saved = g->sssp_cfg;
    double best_ms = 1e300;
    int bd = 0, bt = 256;
    std::string json = "{\"candidates\": [";
    bool first = true;
    for (int d : deltas) {
        for (int t : tiles) {
            int rc = c2g_sssp_set_config(g, d, t, saved.max_iter);
            if (rc) return rc;
            double ms = 0.0;
            bool same = true;
            // one warm-up, then the timed samples
            c2g_stats st;
            if ((rc = c2g_sssp(g, sources[0], use_seeds, seed_mode, dist.data(), 0, &st))) return rc;
            for (int32_t i = 0; i < n; ++i) {
                int32_t* out = first ? ref[i].data() : dist.data();
                if ((rc = c2g_sssp(g, sources[i], use_seeds, seed_mode, out, 0, &st))) return rc;
                ms += st.device_ms;
                if (!first && std::memcmp(out, ref[i].data(), sizeof(int32_t) * (size_t)V) != 0) same = false;
            }
            ms /= n;
            char buf[160];
            snprintf(buf, sizeof(buf), "%s{\"delta\": %d, \"tile\": %d, \"ms_per_query\": %.4f, \"valid\": %s}",
                     first ? "" : ", ", d, t, ms, same ? "true" : "false");
            json += buf;
            if (same && ms < best_ms) {
                best_ms = ms;
                bd = d;
                bt = t;
            }
            first = false;
        }
    }
    char tail[128];
    snprintf(tail, sizeof(tail), "], \"best\": {\"delta\": %d, \"tile\": %d, \"ms_per_query\": %.4f}}\n", bd, bt, best_ms);
    json += tail;
    int rc = c2g_sssp_set_config(g, bd, bt, saved.max_iter);
    if (rc) return rc;
    if (json_path) {
        FILE* f = fopen(json_path, "w");
        if (!f) return fail(C2G_ERR_IO, "cannot write %s", json_path);
        fputs(json.c_str(), f);
        fclose(f);
    }
    if (best_delta) *best_delta = bd;
    if (best_tile) *best_tile = bt;
    return C2G_OK;
}
