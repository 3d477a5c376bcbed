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
//   convert2binary <text> <dir>  utils/convert2binary.cpp:10-137 (text edge list -> origin/)
//
// Standard output follows the reference programs line for line: the dataset path
// (sssp-*, ppr-purn), the Graph constructor's three lines, the device line (sssp-*),
// "test for study how to use cuda", the start banner, the per-launch "csr_v" line
// (ppr-purn), "source = <s>end ------------10" (PPR programs), "gpu runtime: <s> seconds"
// over the 10 launches, the "flag ... iteration_num：<n>" line, ten (SSSP) or eleven (PPR)
// result lines, "源顶点source = <s>" (SSSP), the end banner and the Graph destructor's
// line (src/sssp/purn/Main.cu:24-56,108-123, src/sssp/base/Main.cu:22-100,
// src/ppr/purn/Main.cu:33-136,448, src/ppr/base/Main.cu:38-110,408,
// src/adsorption/w-base/Main.cu:39-113, src/sssp/purn/Graph.h:44-46,61).  Numbers print
// as an ostream prints them (%g for times and floats).  adsorption-base leaves out the
// reference's per-round "act_num" trace.  A missing input prints "file:<f> not exist." to
// stderr and exits 0 (core/io.hpp:27-30); other errors print the message and exit 255,
// as CUDA_ERROR's exit(-1) does (core/Util.cuh:17-24).
//
// Environment: C2G_SEEDS=exact makes sssp-purn use the record->vertex sidecar instead
// of the reference's vertex-indexed hvlist read.  C2G_PRUNE_GPU=<device> makes purn-ppr and
// purn-sssp run their visits on that GPU (c2g_prune_ppr_device, c2g_prune_sssp_device: the
// same files, byte for byte).
#include <unistd.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/c2graph.h"

// The reference's labelled lines (UTF-8, as its sources spell them).
static const char kFlagLine[] = "flag \u5df2\u8bbe\u7f6e\u6210 -1  \u7ec8\u6b62\u6761\u4ef6\u4ee5\u6ee1\u8db3"
                                "\t\titeration_num\uff1a%d\n";
static const char kSourceLine[] = "\u6e90\u9876\u70b9source = %d\n";
static const char kPprBanner[] = "==================== PPR with FORWARD PUSH %s ====================";
static const char kSsspBanner[] = "==================== SSSP with FORWARD PUSH %s ============";

static int die(int rc) {
    const char* msg = c2g_last_error();
    if (rc == C2G_ERR_IO) {
        fprintf(stderr, "%s\n", msg);
        exit(0);
    }
    printf("%s\n", msg);
    exit(255);
}

static c2g_graph* load(const char* dir, int variant) {
    c2g_graph* g = nullptr;
    int rc = c2g_graph_load(dir, variant, 0, &g);
    if (rc) die(rc);
    int32_t V = 0, R = 0;
    int64_t E = 0;
    c2g_graph_info(g, &V, &E, &R);
    printf("INIT--class Graph is constructed\n");
    printf("The vertex num is:%d\n", V);
    printf("The edge num is:%lld\n", (long long)E);
    return g;
}

static void graph_done(c2g_graph* g) {
    c2g_graph_free(g);
    printf("CLEAR--class Graph is destroyed\n");
}

// Two consecutive int32 values of <dir>/<sub>/<name>.bin at index i (row bounds).
static int read_pair(const char* dir, const char* sub, const char* name, int32_t i, int32_t* a, int32_t* b) {
    std::string path = std::string(dir) + "/" + sub + "/" + name + ".bin";
    FILE* f = fopen(path.c_str(), "rb");
    if (!f) return -1;
    int32_t v[2] = {0, 0};
    const bool ok = fseek(f, (long)i * 4, SEEK_SET) == 0 && fread(v, 4, 2, f) == 2;
    fclose(f);
    *a = v[0];
    *b = v[1];
    return ok ? 0 : -1;
}

static int run_sssp(const char* dir, int32_t source, bool pruned) {
    printf("%s\n", dir);
    c2g_graph* g = load(dir, pruned ? C2G_GRAPH_SSSP : C2G_GRAPH_ORIGIN);
    int ndev = 0;
    c2g_device_count(&ndev);
    printf(ndev > 0 ? "Using GPU device 0\n" : "No GPU available, falling back to CPU\n");
    printf("test for study how to use cuda\n");
    const char* env = getenv("C2G_SEEDS");
    const int mode = (env && strcmp(env, "exact") == 0) ? C2G_SEEDS_EXACT : C2G_SEEDS_COMPAT;
    int32_t s = source;
    int rc;
    if ((rc = c2g_sssp_resolve_source(g, source, pruned ? 1 : 0, mode, &s))) die(rc);
    int32_t V = 0;
    c2g_graph_info(g, &V, nullptr, nullptr);
    std::vector<int32_t> dist((size_t)V);
    printf("\n");
    printf(kSsspBanner, "starts");
    printf("\n");
    c2g_stats st;
    double total_ms = 0.0;
    for (int i = 0; i < 10; ++i) {  // the reference times 10 launches on one source
        if ((rc = c2g_sssp(g, s, pruned ? 1 : 0, mode, dist.data(), 0, &st))) die(rc);
        total_ms += st.device_ms;
    }
    if (!pruned) {
        printf("\n");
        printf(kSsspBanner, "ends");
        printf("\n");
    }
    printf(kFlagLine, st.iterations);
    for (int i = 0; i < 10 && i < V; ++i) printf("%d\t%d\n", i, dist[i]);
    printf("gpu runtime: %g seconds\n", total_ms / 1000.0);
    printf(kSourceLine, s);
    graph_done(g);
    return 0;
}

static int run_ppr(const char* dir, int32_t source, bool pruned, bool adsorption) {
    if (pruned) printf("%s\n", dir);
    c2g_graph* g = load(dir, pruned ? C2G_GRAPH_PPR : C2G_GRAPH_ORIGIN);
    printf("test for study how to use cuda\n");
    int32_t V = 0;
    c2g_graph_info(g, &V, nullptr, nullptr);
    if (source < 0 || source >= V) {
        printf("source %d out of range\n", source);
        return 255;
    }
    c2g_ppr_params p;
    c2g_ppr_default_params(g, adsorption ? 1 : 0, &p);
    std::vector<float> pr((size_t)V), res((size_t)V);
    printf("\n");
    printf(kPprBanner, "starts");
    printf("\n");
    int32_t h0 = 0, h1 = 0, v0 = 0, v1 = 0;
    if (pruned && (read_pair(dir, "ppr", "hvlist", source, &h0, &h1) || read_pair(dir, "ppr", "vlist", source, &v0, &v1)))
        die(C2G_ERR_IO);
    c2g_stats st;
    double total_ms = 0.0;
    for (int i = 0; i < 10; ++i) {
        if (pruned) printf("csr_v %d--%d\n", h1 - h0, v1 - v0);
        int rc = c2g_ppr(g, source, &p, pr.data(), res.data(), 0, &st);
        if (rc) die(rc);
        total_ms += st.device_ms;
    }
    printf("source = %dend ------------10\n", source);
    printf("gpu runtime: %g seconds\n", total_ms / 1000.0);
    printf(kFlagLine, st.iterations);
    printf(kPprBanner, "ends");
    printf("\n\n");
    for (int i = 0; i <= 10 && i < V; ++i)
        printf("%d.\tpagerank\t %g\tresidual\t%g\n", i, (double)pr[i], (double)res[i]);
    graph_done(g);
    return 0;
}

// convert2binary <text> <dir> (utils/convert2binary.cpp:10-137): the reference's four lines
// on stdout; an unreadable input prints the reference's message and exits 0 (the reference
// then writes an empty graph; nothing is written here).
static int run_convert(const char* text, const char* dir) {
    printf("Reading graph from %s\n", text);
    int64_t mv = 0, V = 0, E = 0;
    const int rc = c2g_convert_text(text, dir, &mv, &V, &E);
    if (rc == C2G_ERR_IO && access(text, R_OK) != 0) {
        fprintf(stderr, "Error opening file: %s\n", text);
        return 0;
    }
    if (rc) die(rc);
    printf("Max Vertex Number: %lld\n", (long long)mv);
    printf("Vertex Number: %lld\n", (long long)V);
    printf("Edge Number: %lld\n", (long long)E);
    return 0;
}

static int run_prune(const char* dir, bool ppr) {
    auto t0 = std::chrono::steady_clock::now();
    const char* gpu = getenv("C2G_PRUNE_GPU");
    int rc;
    if (ppr && gpu && *gpu)  // alpha 0.2: the reference's baked factor 0.8 (1 - 0.2 is the same double)
        rc = c2g_prune_ppr_device(dir, 0.2, atoi(gpu), nullptr, nullptr, nullptr);
    else if (gpu && *gpu)
        rc = c2g_prune_sssp_device(dir, atoi(gpu), nullptr, nullptr, nullptr);
    else
        rc = ppr ? c2g_prune_ppr(dir) : c2g_prune_sssp(dir);
    if (rc) die(rc);
    const double s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    fprintf(stderr, "Filter time : %.4f(s)\n", s);
    return 0;
}

int main(int argc, char** argv) {
    std::string prog = argv[0];
    const size_t slash = prog.find_last_of('/');
    if (slash != std::string::npos) prog = prog.substr(slash + 1);
    if (prog == "convert2binary") {
        if (argc != 3) {
            fprintf(stderr, "Usage: %s <edge_list.txt> <dataset_dir>\n", prog.c_str());
            return 0;
        }
        return run_convert(argv[1], argv[2]);
    }
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
