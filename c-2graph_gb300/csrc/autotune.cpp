// Autotuner of the SSSP kernel's tile and bucket (near/far delta) parameters.
//
// The reference hard-codes its launch geometry (core/Util.cuh:31-34) and has no bucket
// parameter.  Here the best (delta, tile) depends on the graph's weight range and degree
// skew, so c2g_sssp_autotune times every candidate on sample sources.  A candidate whose
// distances differ from the first candidate's is rejected (all must be the same
// fixed point).  The winner is applied to the handle and, when a path is given, written
// as a JSON record of every timing.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include <cuda_runtime.h>

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

// Autotuner of the batched SSSP's expansion tiles (c2g_sssp_batch_set_tile) and round
// shape (c2g_sssp_batch_set_pull): the size of the big tiles and the per-warp tile count
// above which a round walks them, then, at the chosen tiles, the relaxation share above
// which a round pulls over the reverse CSR.  Big tiles cut the tile-queue traffic and the
// owner lookups of long rounds; small ones balance the short rounds; pull rounds pay in
// the rounds where most queries of most active words are active.  Which settings are best
// depends on the batch (queries, graph, weights), so c2g_sssp_batch_autotune times each
// candidate on the caller's batch (one warm-up launch, then `reps` timed ones; the batch
// kernel's device time).  A candidate whose distances differ from the first candidate's
// on any of the first 8 queries is rejected (every candidate must reach the same fixed
// point).  The winners are applied to the handle and, when a path is given, written as a
// JSON record of every timing.
extern "C" int c2g_sssp_batch_autotune(c2g_graph* g, int32_t n, const int32_t* sources, int use_seeds,
                                       int seed_mode, int32_t reps, const char* json_path, int32_t* best_big_steps,
                                       int32_t* best_min_tiles) {
    using namespace c2g;
    if (!g || !sources || n < 1) return fail(C2G_ERR_ARG, "autotune: need a batch of sources");
    if (reps < 1) reps = 1;
    struct Cand {
        int big, min;
        float frac;
    };
    int32_t saved_big = 512, saved_min = 16;
    c2g_sssp_batch_get_tile(g, &saved_big, &saved_min);
    float saved_frac = 0.3f;
    c2g_sssp_batch_get_pull(g, &saved_frac);
    std::vector<Cand> tiles = {{128, 1, saved_frac}};
    for (int big : {256, 512, 1024, 2048})
        for (int mn : {4, 16, 64}) tiles.push_back({big, mn, saved_frac});
    const size_t V = (size_t)g->V, rows = (size_t)(n < 8 ? n : 8);
    int32_t* dd = nullptr;
    {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(g->device);
        const cudaError_t e = cudaMalloc(&dd, sizeof(int32_t) * V * (size_t)n);
        if (prev >= 0) cudaSetDevice(prev);
        if (e != cudaSuccess) return fail(C2G_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
    }
    std::vector<int32_t> ref(rows * V), got(rows * V);
    double best_ms = 1e300;
    Cand best{saved_big, saved_min, saved_frac};
    std::string json = "{\"candidates\": [";
    int rc = C2G_OK;
    bool first = true;
    // one candidate: applied, timed and checked; the fastest valid one becomes `best`
    auto run = [&](const Cand& c) {
        if ((rc = c2g_sssp_batch_set_tile(g, c.big, c.min)) || (rc = c2g_sssp_batch_set_pull(g, c.frac))) return;
        c2g_stats st;
        double ms = 0.0;
        for (int k = 0; k <= reps && !rc; ++k) {
            rc = c2g_sssp_batch(g, n, sources, use_seeds, seed_mode, dd, 1, C2G_LAYOUT_QUERY_MAJOR, &st);
            if (k > 0) ms += st.device_ms;
        }
        if (rc) return;
        ms /= reps;
        int32_t* dst = first ? ref.data() : got.data();
        if (cudaMemcpy(dst, dd, sizeof(int32_t) * rows * V, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = fail(C2G_ERR_CUDA, "autotune: copying results failed");
            return;
        }
        const bool same = first || std::memcmp(got.data(), ref.data(), sizeof(int32_t) * rows * V) == 0;
        const bool valid = same && st.status_flags == 0;
        char buf[224];
        snprintf(buf, sizeof(buf),
                 "%s{\"big_steps\": %d, \"min_tiles_per_warp\": %d, \"pull_frac\": %g, \"ms_per_batch\": %.3f, "
                 "\"valid\": %s}",
                 first ? "" : ", ", c.big, c.min, (double)c.frac, ms, valid ? "true" : "false");
        json += buf;
        if (valid && ms < best_ms) {
            best_ms = ms;
            best = c;
        }
        first = false;
    };
    for (const Cand& c : tiles) {
        run(c);
        if (rc) break;
    }
    if (!rc) {  // the round shape at the chosen tiles
        const Cand tiled = best;
        for (float f : {-1.f, 0.15f, 0.3f, 0.5f, 0.75f}) {
            if (f == tiled.frac) continue;  // timed with the tiles
            run({tiled.big, tiled.min, f});
            if (rc) break;
        }
    }
    cudaFree(dd);
    if (rc) {
        c2g_sssp_batch_set_tile(g, saved_big, saved_min);
        c2g_sssp_batch_set_pull(g, saved_frac);
        return rc;
    }
    char tail[192];
    snprintf(tail, sizeof(tail),
             "], \"best\": {\"big_steps\": %d, \"min_tiles_per_warp\": %d, \"pull_frac\": %g, \"ms_per_batch\": %.3f}}\n",
             best.big, best.min, (double)best.frac, best_ms);
    json += tail;
    if ((rc = c2g_sssp_batch_set_tile(g, best.big, best.min)) || (rc = c2g_sssp_batch_set_pull(g, best.frac)))
        return rc;
    if (json_path) {
        FILE* f = fopen(json_path, "w");
        if (!f) return fail(C2G_ERR_IO, "cannot write %s", json_path);
        fputs(json.c_str(), f);
        fclose(f);
    }
    if (best_big_steps) *best_big_steps = best.big;
    if (best_min_tiles) *best_min_tiles = best.min;
    return C2G_OK;
}

// Autotuner of the batched push's round shape: the push-count ratio above which a round
// pulls over the reverse CSR (c2g_ppr_batch_set_pull).  The best ratio depends on how
// dense the batch's rounds get (queries, graph, rmax), so c2g_ppr_batch_autotune times
// each candidate on the caller's batch (one warm-up launch, then `reps` timed ones; the
// batch kernel's device time).  The first candidate is push only; a candidate whose pr
// differs from it by more than the parity bar (L1 1e-6 per query, on the first 8
// queries) is rejected.  The winner is applied to the handle and, when a path is given,
// written as a JSON record of every timing.
extern "C" int c2g_ppr_batch_autotune(c2g_graph* g, int32_t n, const int32_t* sources,
                                      const c2g_ppr_params* params, int32_t reps, const char* json_path,
                                      float* best_ratio) {
    using namespace c2g;
    if (!g || !sources || !params || n < 1) return fail(C2G_ERR_ARG, "autotune: need a batch of sources");
    if (reps < 1) reps = 1;
    const float ratios[] = {-1.f, 1.f, 2.f, 4.f, 8.f, 16.f, 32.f};
    const size_t V = (size_t)g->V, rows = (size_t)(n < 8 ? n : 8);
    float* dpr = nullptr;
    {
        int prev = -1;
        cudaGetDevice(&prev);
        cudaSetDevice(g->device);
        const cudaError_t e = cudaMalloc(&dpr, sizeof(float) * V * (size_t)n);
        if (prev >= 0) cudaSetDevice(prev);
        if (e != cudaSuccess) return fail(C2G_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
    }
    std::vector<float> ref(rows * V), got(rows * V);
    const float saved = g->ppr_cfg.batch_pull_ratio;
    double best_ms = 1e300;
    float best = saved;
    std::string json = "{\"candidates\": [";
    int rc = C2G_OK;
    bool first = true;
    for (float r : ratios) {
        if ((rc = c2g_ppr_batch_set_pull(g, r))) break;
        c2g_stats st;
        double ms = 0.0;
        for (int k = 0; k <= reps && !rc; ++k) {
            rc = c2g_ppr_batch(g, n, sources, params, dpr, nullptr, 1, C2G_LAYOUT_QUERY_MAJOR, &st);
            if (k > 0) ms += st.device_ms;
        }
        if (rc) break;
        ms /= reps;
        float* dst = first ? ref.data() : got.data();
        if (cudaMemcpy(dst, dpr, sizeof(float) * rows * V, cudaMemcpyDeviceToHost) != cudaSuccess) {
            rc = fail(C2G_ERR_CUDA, "autotune: copying results failed");
            break;
        }
        double worst = 0.0;
        if (!first)
            for (size_t q = 0; q < rows; ++q) {
                double l1 = 0.0;
                for (size_t v = 0; v < V; ++v) l1 += std::fabs((double)got[q * V + v] - (double)ref[q * V + v]);
                worst = l1 > worst ? l1 : worst;
            }
        const bool valid = worst <= 1e-6 && st.status_flags == 0;
        char buf[192];
        snprintf(buf, sizeof(buf), "%s{\"ratio\": %g, \"ms_per_batch\": %.3f, \"l1_vs_push\": %.3g, \"valid\": %s}",
                 first ? "" : ", ", (double)r, ms, worst, valid ? "true" : "false");
        json += buf;
        if (valid && ms < best_ms) {
            best_ms = ms;
            best = r;
        }
        first = false;
    }
    cudaFree(dpr);
    if (rc) {
        c2g_ppr_batch_set_pull(g, saved);
        return rc;
    }
    char tail[128];
    snprintf(tail, sizeof(tail), "], \"best\": {\"ratio\": %g, \"ms_per_batch\": %.3f}}\n", (double)best, best_ms);
    json += tail;
    if ((rc = c2g_ppr_batch_set_pull(g, best))) return rc;
    if (json_path) {
        FILE* f = fopen(json_path, "w");
        if (!f) return fail(C2G_ERR_IO, "cannot write %s", json_path);
        fputs(json.c_str(), f);
        fclose(f);
    }
    if (best_ratio) *best_ratio = best;
    return C2G_OK;
}
