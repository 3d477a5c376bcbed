// Drop-in command-line programs with the reference's signatures, thin callers of the
// C ABI.  One binary; the program is chosen by the name it is invoked under:
//
//   sssp-base <dir> <source>   src/sssp/base/Main.cu:16-103  (origin/, 10 launches)
//   sssp-purn <dir> <source>   src/sssp/purn/Main.cu:18-126  (sssp/ + record seeds)
//   ppr-base  <dir> <source>   src/ppr/base/Main.cu:25-118   (origin/ flist)
//   ppr-purn  <dir> <source>   src/ppr/purn/Main.cu:26-145   (ppr/ + record seeds)
//   adsorption-base <dir> <source>  src/adsorption/w-base/Main.cu (origin/ flist)
//   purn-sssp <dir>            src/purn-sssp.cpp:61-352
//   purn-ppr  <dir>            src/purn-ppr.cpp:63-344
//
// Output lines kept from the reference: the dataset path, graph sizes, the iteration
// count, ten "i<TAB>value" result lines, "gpu runtime: <s> seconds" (all 10 launches),
// and the adjusted source.  A missing input prints "file:<f> not exist." to stderr and
// exits 0 (core/io.hpp:27-30); other errors print the message and exit 255, as
// CUDA_ERROR's exit(-1) does (core/Util.cuh:17-24).
//
// Environment: C2G_SEEDS=exact makes sssp-purn use the record->vertex sidecar instead
// of the reference's vertex-indexed hvlist read.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/c2graph.h"

static int die(int rc) {
    const char* msg = c2g_last_error();
    if (rc == C2G_ERR_IO) {
        fprintf(stderr, "%s\n", msg);
        exit(0);
    }
    printf("%s\n", msg);
    exit(255);
}

static void print_graph(c2g_graph* g) {
    int32_t V = 0, R = 0;
    int64_t E = 0;
    c2g_graph_info(g, &V, &E, &R);
    printf("INIT--class Graph is constructed\n");
    printf("The vertex num is:%d\n", V);
    printf("The edge num is:%lld\n", (long long)E);
}

static int run_sssp(const char* dir, int32_t source, bool pruned) {
    printf("%s\n", dir);
    c2g_graph* g = nullptr;
    int rc = c2g_graph_load(dir, pruned ? C2G_GRAPH_SSSP : C2G_GRAPH_ORIGIN, 0, &g);
    if (rc) die(rc);
    print_graph(g);
    const char* env = getenv("C2G_SEEDS");
    const int mode = (env && strcmp(env, "exact") == 0) ? C2G_SEEDS_EXACT : C2G_SEEDS_COMPAT;
    int32_t s = source;
    if ((rc = c2g_sssp_resolve_source(g, source, pruned ? 1 : 0, mode, &s))) die(rc);
    int32_t V = 0;
    c2g_graph_info(g, &V, nullptr, nullptr);
    std::vector<int32_t> dist((size_t)V);
    printf("\n==================== SSSP with FORWARD PUSH starts ============\n");
    c2g_stats st;
    double total_ms = 0.0;
    for (int i = 0; i < 10; ++i) {  // the reference times 10 launches on one source
        if ((rc = c2g_sssp(g, s, pruned ? 1 : 0, mode, dist.data(), 0, &st))) die(rc);
        total_ms += st.device_ms;
    }
    printf("iteration_num:%d\n", st.iterations);
    for (int i = 0; i < 10 && i < V; ++i) printf("%d\t%d\n", i, dist[i]);
    printf("gpu runtime: %g seconds\n", total_ms / 1000.0);
    printf("source = %d\n", s);
    c2g_graph_free(g);
    return 0;
}

static int run_ppr(const char* dir, int32_t source, bool pruned, bool adsorption) {
    printf("%s\n", dir);
    c2g_graph* g = nullptr;
    int rc = c2g_graph_load(dir, pruned ? C2G_GRAPH_PPR : C2G_GRAPH_ORIGIN, 0, &g);
    if (rc) die(rc);
    print_graph(g);
    int32_t V = 0;
    c2g_graph_info(g, &V, nullptr, nullptr);
    if (source < 0 || source >= V) {
        printf("source %d out of range\n", source);
        return 255;
    }
    c2g_ppr_params p;
    c2g_ppr_default_params(g, adsorption ? 1 : 0, &p);
    std::vector<float> pr((size_t)V), res((size_t)V);
    printf("\n==================== PPR with FORWARD PUSH starts ====================\n");
    c2g_stats st;
    double total_ms = 0.0;
    for (int i = 0; i < 10; ++i) {
        if ((rc = c2g_ppr(g, source, &p, pr.data(), res.data(), 0, &st))) die(rc);
        total_ms += st.device_ms;
    }
    printf("source = %d end ------------10\n", source);
    printf("gpu runtime: %g seconds\n", total_ms / 1000.0);
    printf("iteration_num:%d\n", st.iterations);
    printf("==================== PPR with FORWARD PUSH ends ====================\n\n");
    for (int i = 0; i <= 10 && i < V; ++i) printf("%d.\tpagerank\t %g\tresidual\t%g\n", i, pr[i], res[i]);
    c2g_graph_free(g);
    return 0;
}

static int run_prune(const char* dir, bool ppr) {
    auto t0 = std::chrono::steady_clock::now();
    int rc = ppr ? c2g_prune_ppr(dir) : c2g_prune_sssp(dir);
    if (rc) die(rc);
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    fprintf(stderr, "Filter time : %.4f(s)\n", s);
    return 0;
}

int main(int argc, char** argv) {
    std::string prog = argv[0];
    const size_t slash = prog.find_last_of('/');
    if (slash != std::string::npos) prog = prog.substr(slash + 1);
    if (prog == "purn-sssp" || prog == "purn-ppr") {
        if (argc != 2) {
            fprintf(stderr, "Usage: %s <dataset_dir>\n", prog.c_str());
            return 0;
        }
        return run_prune(argv[1], prog == "purn-ppr");
    }
    if (argc < 3) {
        fprintf(stderr, "Usage: %s <dataset_dir> <source>\n", prog.c_str());
        return 2;
    }
    const char* dir = argv[1];
    const int32_t source = (int32_t)atoi(argv[2]);
    if (prog == "sssp-base") return run_sssp(dir, source, false);
    if (prog == "sssp-purn") return run_sssp(dir, source, true);
    if (prog == "ppr-base") return run_ppr(dir, source, false, false);
    if (prog == "ppr-purn") return run_ppr(dir, source, true, false);
    if (prog == "adsorption-base") return run_ppr(dir, source, false, true);
    fprintf(stderr, "unknown program name %s\n", prog.c_str());
    return 2;
}
