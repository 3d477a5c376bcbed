// Internal host-side types of the C^2graph GB300 library (not part of the ABI).
//
// Device layout of a graph (HBM):
//   row   int32[V+1]        CSR row pointer (reference vlist)
//   adj_w int2[E]           (target, int32 weight) interleaved: one 8-byte load per edge
//   adj_f int2[E]           (target, float weight bits) for the push kernels
//   hv/he/hw                pruned records (reference hvlist/helist/hwlist)
//   rec_of_vertex int32[V]  vertex -> record index (from the hvmap sidecar), -1 if none
// Per-query workspaces are allocated on first use and kept for the handle's lifetime.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <vector>

#include "../../include/c2graph.h"
#include "host_io.h"

namespace c2g {

#define C2G_CUDA(call)                                                                       \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return ::c2g::fail(e_ == cudaErrorMemoryAllocation ? C2G_ERR_OOM : C2G_ERR_CUDA, \
                               "%s in %s at line %d", cudaGetErrorString(e_), __FILE__,      \
                               __LINE__);                                                    \
    } while (0)

// Control block of one persistent traversal launch; zeroed before every launch.
struct TraversalCtl {
    unsigned long long qctr[3];  // frontier counters per round slot: (count<<32)|edges
    unsigned tilectr[3];         // dynamic tile scheduler per round slot
    unsigned listctr[3];         // PPR touched-list counters per round slot
    unsigned dctr[3];            // PPR activated vertices without out-edges, per slot
    unsigned farctr[3];          // SSSP far piles (rotating: current, target, free)
    int farmin[3];
    unsigned bar_count, bar_gen;  // GridBarrier
    int flags;                    // C2G_FLAG_*
    int iterations;
    long long popped, relaxed, touched, seeds;
    int pad[1];
    unsigned long long phase_ns[4];  // block 0's time per phase (see phase_mark)
    unsigned long long pcount[3];    // batched PPR: (query, edge) pushes of the frontier per round slot
};

// Per-round trace of a batched launch (c2g_graph_last_rounds): the device time at the
// start of each round (block 0, right after the grid barrier that ends the previous
// round), the round's work units and its shape; the entry after the last round holds the
// end time.
constexpr int kMaxTraceRounds = 1024;
struct RoundTrace {
    unsigned long long t_ns;
    long long work;  // PPR: (query, edge) pushes of the round; SSSP: edge-word steps
    int shape;       // 1 pull round, 0 push (PPR) or expansion (SSSP) round
    unsigned mid_ns;  // from the round's start to the end of its first phase (expansion / push or pull)
};

// Stamps survive across launches; the kernel advances the bases itself.
struct StampState {
    int stamp_base;
    int epoch_base;
    int pad[2];
};

struct SsspWork {
    int* dist = nullptr;
    int* stamp = nullptr;
    int* farstamp = nullptr;
    int2* q[2] = {nullptr, nullptr};
    int* mark[2] = {nullptr, nullptr};
    int* far = nullptr;  // three far piles of V ids each
    unsigned* bits = nullptr;  // next-frontier bitmap of the Bellman-Ford kernel (V/32 words)
    TraversalCtl* ctl = nullptr;
    StampState* st = nullptr;
    unsigned mark_cap = 0;
    int log_tile = -1;
};

struct PprWork {
    float* pr = nullptr;
    double* res = nullptr;
    double* msg = nullptr;
    double* qd = nullptr;
    float* res_f = nullptr;  // residual as float for the caller
    int* stamp = nullptr;
    int2* q[2] = {nullptr, nullptr};
    double* qval[2] = {nullptr, nullptr};
    int* mark[2] = {nullptr, nullptr};
    int* touched = nullptr;
    int* dangle = nullptr;
    TraversalCtl* ctl = nullptr;
    StampState* st = nullptr;
    unsigned mark_cap = 0;
    int log_tile = -1;
};

struct SsspConfig {
    int delta = 0;       // <= 0: no near/far split
    int log_tile = 8;    // 256 edges per warp tile
    int max_iter = 1 << 20;
    int batch_tile_big_log = 9;  // batched expansion: 512 edge-word steps per big tile
    int batch_tile_min_log = 4;  // ... in rounds with at least 16 big tiles per warp
    float batch_pull_frac = 0.3f;  // batched rounds with more (query, edge) relaxations than this * E * Q
                                   // pull over the reverse CSR (< 0: never)
};

struct PprConfig {
    float batch_pull_ratio = 8.0f;  // batched rounds with more than ratio * E pushes pull (< 0: never)
    int log_tile = 8;
    int pull_div = 0;   // pull round when frontier out-edges * pull_div > E; 0 = push only (default)
    int dense_div = 16;  // dense push round (red.add, apply sweep over V) when out-edges * dense_div > E
};

constexpr int kPullTileLog = 8;  // in-edges per pull tile (reverse-CSR markers)

struct LaunchGeom {
    int blocks = 0;
    int threads = 512;
};

}  // namespace c2g

struct c2g_graph {
    int device = 0;
    int variant = 0;
    int32_t V = 0;
    int64_t E = 0;
    int32_t* row = nullptr;
    int2* adj_w = nullptr;
    int2* adj_f = nullptr;
    int32_t* row_r = nullptr;  // reverse CSR with float weights (pull rounds, adjoint), on demand
    int2* adj_r = nullptr;
    int2* adj_rw = nullptr;     // the same in-edges with int32 weights (batched SSSP pull rounds), on
                                // demand; adj_r itself when the graph has no float weights
    int32_t* mark_r = nullptr;  // pull-tile owner markers over row_r
    int32_t* mark_f = nullptr;  // pull-tile owner markers over row (pulls on the reverse graph)
    // pruned records
    int32_t R = -1;
    int64_t H = 0;
    int32_t* hv = nullptr;
    int32_t* he = nullptr;
    int32_t* hw = nullptr;  // int32 or float bits
    bool hw_float = false;
    int32_t* rec_of_vertex = nullptr;
    // host copies needed for source rules and seed ranges
    std::vector<int32_t> h_row;
    std::vector<int32_t> h_hv;
    std::vector<int32_t> h_rec_of_vertex;
    std::vector<int32_t> h_he, h_hw;  // record targets / weights (bits)
    void* batch = nullptr;            // batched-query workspaces (batch.cu)
    void* ppr_batch = nullptr;
    void* ads = nullptr;              // label-propagation workspace (adsorption.cu)
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    std::mutex mu;
    c2g::SsspConfig sssp_cfg;
    c2g::PprConfig ppr_cfg;
    c2g::SsspWork sssp;
    c2g::PprWork ppr;
    c2g::LaunchGeom geom_sssp, geom_ppr, geom_bits;
    int num_sms = 0;
    float grid_scale = 1.0f;  // fraction of the GPU a batched launch may occupy
    unsigned long long barrier_ns = 0;  // grid-barrier wait limit (0: per-kernel default)
    unsigned long long last_phase_ns[4] = {0, 0, 0, 0};  // phases of the last launch
    // float-weight statistics (batched pull rounds), valid = false until computed: the
    // largest positive weight (bits)
    bool wstat_valid = false;
    uint32_t wstat_wmax_bits = 0;
    int stall_next_sssp = 0;            // failure-detection test: next SSSP barrier cannot complete
    c2g::RoundTrace* last_trace = nullptr;  // device trace of the last batched launch (in its workspace)
    bool borrowed = false;    // a view: graph arrays belong to another handle
};

namespace c2g {

// Kernel launchers (sssp.cu / ppr.cu).  All work is issued on g->stream.
int sssp_launch(c2g_graph* g, int32_t source, const int32_t* seed_v, const int32_t* seed_w,
                int32_t n_seeds, int32_t* dist_dev, float* ms);
int ppr_launch(c2g_graph* g, int32_t source, const c2g_ppr_params& p, const int32_t* seed_v,
               const float* seed_w, int32_t n_seeds, float* pr_dev, float* res_dev, float* ms);
int ppr_launch_view(c2g_graph* g, const int32_t* row, const int2* adj, const int32_t* row_rev, const int2* adj_rev,
                    const int32_t* mark_rev, int32_t source, const c2g_ppr_params& pp, float absorb, int32_t n_src,
                    const int32_t* src_list, const float* src_r0, const int32_t* seed_v, const float* seed_w,
                    int32_t n_rec, float* pr_dev, float* res_dev, float* ms);
int build_markers(c2g_graph* g, const int* row, int** out);
void sssp_free(c2g_graph* g);
void ppr_free(c2g_graph* g);
// A handle sharing `base`'s device graph arrays with its own stream, workspaces and lock.
int graph_view(c2g_graph* base, c2g_graph** out);
void batch_free(c2g_graph* g);
void ppr_batch_free(c2g_graph* g);
void ads_free(c2g_graph* g);
int build_reverse_graph(c2g_graph* g);
// The reverse CSR's in-edges with int32 weights (batched SSSP pull rounds).
int build_reverse_int(c2g_graph* g);
// Reverse CSR and the weight statistics of the batched pull rounds (once per weights).
int ppr_pull_prepare(c2g_graph* g);
int ppr_batch_launch(c2g_graph* g, int32_t nq, const int32_t* sources, const c2g_ppr_params& prm,
                     const std::vector<int32_t>* seed_off, const std::vector<int32_t>* seed_v,
                     const std::vector<float>* seed_w, float* pr_out, float* res_out, int on_device, int query_major,
                     float* ms, long long* counters, TraversalCtl* ctl_out);
// Resident batches (session.cu): workspaces of Q slots that keep their state between
// launches, and one epoch (at most `rounds` rounds) of the batched kernels over them.
struct PprBatchArrays {
    float* pr;
    double* res;
    double* rq[2];
    float2* rqf[2];
    unsigned* amask[2];
    unsigned* dmask;
};
void session_set_grid_share(c2g_session* s, float share);
int sssp_batch_reserve(c2g_graph* g, int Q, int** dist, unsigned** mask);
int sssp_batch_epoch(c2g_graph* g, int Q, int rounds, float* ms, long long* counters, TraversalCtl* ctl_out);
int ppr_batch_reserve(c2g_graph* g, int Q, PprBatchArrays* a);
int ppr_batch_epoch(c2g_graph* g, int Q, const c2g_ppr_params& prm, int cur0, int rounds, float* ms,
                    long long* counters, TraversalCtl* ctl_out);
int sssp_batch_launch(c2g_graph* g, int32_t nq, const int32_t* sources, const std::vector<int32_t>* seed_off,
                      const std::vector<int32_t>* seed_v, const std::vector<int32_t>* seed_w, int32_t* out,
                      int out_on_device, int query_major, float* ms, long long* counters, TraversalCtl* ctl_out);

}  // namespace c2g
