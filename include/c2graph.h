/*
 * c2graph.h - C ABI of the GB300 (sm_103a) implementation of C^2graph's weighted
 * traversal path: SSSP relaxation on the original or pruned CSR, PPR forward push,
 * adsorption, and the offline C^2graph-P pruners that produce the pruned CSR.
 *
 * The reference (lihuaibei7951/C-2graph) has no library API; its boundary is a set of
 * command-line programs.  Each entry point below names the reference code it replaces
 * (file:line in the reference project).  The drop-in programs sssp-base, sssp-purn,
 * ppr-purn, ppr-base, purn-sssp and purn-ppr are thin callers of this ABI.
 *
 * Conventions
 *   - Every function returns int status: C2G_OK (0) or a negative C2G_ERR_* code.
 *     Nothing here calls exit(); c2g_last_error() gives a message for the calling thread.
 *   - Output buffers are owned by the caller.  A flag says whether a pointer is host
 *     memory or device memory of the graph's device.
 *   - A graph handle owns its device CSR and its per-query workspace, and issues all
 *     work on one CUDA stream.  Calls on one handle are serialised by the handle;
 *     distinct handles may be used from distinct threads.
 *   - Binary files use the reference layout: raw little-endian int32/float32 arrays
 *     with no header (reference core/io.hpp:25-40).
 */
#ifndef C2GRAPH_H
#define C2GRAPH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define C2G_ABI_VERSION 2

/* ---- status codes --------------------------------------------------------------- */
#define C2G_OK               0
#define C2G_ERR_ARG         -1  /* null pointer, bad enum, bad parameter               */
#define C2G_ERR_IO          -2  /* file missing, unreadable or short                    */
#define C2G_ERR_FORMAT      -3  /* arrays inconsistent (vlist not monotone, bad ids)    */
#define C2G_ERR_CUDA        -4  /* CUDA runtime error                                   */
#define C2G_ERR_OOM         -5  /* device or host allocation failed                     */
#define C2G_ERR_RANGE       -6  /* source out of range, or no eligible source           */
#define C2G_ERR_TIMEOUT     -7  /* a bounded device-side wait ran out                   */
#define C2G_ERR_OVERFLOW    -8  /* a device queue would overflow                        */
#define C2G_ERR_UNSUPPORTED -9  /* graph variant lacks what the call needs             */
#define C2G_ERR_NODEVICE   -10  /* no CUDA device                                       */

/* device-side status bits reported in c2g_stats.status_flags */
#define C2G_FLAG_BARRIER_TIMEOUT  0x1  /* a grid barrier wait ran out                   */
#define C2G_FLAG_ITER_CAP         0x2  /* the iteration cap stopped the traversal       */
#define C2G_FLAG_QUEUE_OVERFLOW   0x4  /* a queue append was dropped                    */
#define C2G_FLAG_BOUNDS           0x8  /* an index check failed; the access was skipped */

/* which directory of a dataset a graph is read from */
typedef enum {
    C2G_GRAPH_ORIGIN = 0, /* <dir>/origin/{vlist,elist,wlist[,flist]}.bin               */
    C2G_GRAPH_SSSP   = 1, /* <dir>/sssp/{vlist,elist,wlist,hvlist,helist,hwlist}.bin    */
    C2G_GRAPH_PPR    = 2  /* <dir>/ppr/{vlist,elist,wlist(float),hvlist,helist,hwlist}  */
} c2g_variant;

/* How sssp-purn picks the pruned-record seeds of a source.
 *   COMPAT: hvlist is indexed by the source id, exactly as the reference does
 *           (src/sssp/purn/Main.cu:68-79), although purn-sssp writes one record per
 *           pruned vertex in pruning order (src/purn-sssp.cpp:279-286).
 *   EXACT:  the record that belongs to the source is found through the record->vertex
 *           sidecar (sssp/hvmap.bin) written by c2g_prune_sssp. */
typedef enum { C2G_SEEDS_COMPAT = 0, C2G_SEEDS_EXACT = 1 } c2g_seed_mode;

typedef struct c2g_graph c2g_graph;

/* per-call statistics (device counters, read back after the call) */
typedef struct c2g_stats {
    int32_t source;          /* source actually traversed                              */
    int32_t iterations;      /* frontier rounds executed (reference iteration_num)     */
    int64_t vertices_popped; /* sum over rounds of frontier vertices expanded          */
    int64_t edges_relaxed;   /* sum over rounds of frontier out-edges relaxed/pushed   */
    int64_t touched;         /* PPR: sum over rounds of vertices that got a message    */
    int64_t n_seeds;         /* seed entries applied before the first round            */
    double  alg_bytes;       /* algorithmic bytes of the call (byte model per path)    */
    float   device_ms;       /* device time of the traversal launch (CUDA events)      */
    int32_t status_flags;    /* C2G_FLAG_* bits, 0 when clean                          */
    int32_t reserved;
} c2g_stats;

/* PPR / adsorption push parameters (reference src/ppr/purn/Main.cu:66-67,
 * src/ppr/base/Main.cu:61-62, src/adsorption/w-base/Main.cu:63-64,149-152). */
typedef struct c2g_ppr_params {
    float   alpha;    /* teleport probability: pr += alpha*r, push (1-alpha)*r*w      */
    float   rmax;     /* activation threshold: a vertex is pushed when residual > rmax */
    float   r0;       /* base mode: residual placed on the source                     */
    float   pr0;      /* base mode: value added to pr[source] before the first round  */
    int32_t max_iter; /* round cap (reference: 500 for PPR, 2000 for adsorption)       */
    int32_t seeded;   /* 0: base init (src/ppr/base/Main.cu:146-150)
                         1: pruned-graph init with host-side first hop
                            (src/ppr/purn/Main.cu:78-101,173-198)                    */
} c2g_ppr_params;

/* ---- library ---------------------------------------------------------------------- */
int         c2g_abi_version(void);
const char* c2g_last_error(void);
int         c2g_device_count(int* count);

/* ---- graphs ------------------------------------------------------------------------ */
/* Load <dir>/{origin|sssp|ppr}/ into device memory of `device`.
 * Replaces Graph ctors src/sssp/base/Graph.h:30-51, src/sssp/purn/Graph.h:33-48,
 * src/ppr/purn/Graph.h:34-46 and DeviceMemory::CudaMemcpyGraph
 * (src/sssp/purn/DeviceMemory.cuh:48-67).  A missing file is C2G_ERR_IO (the
 * reference prints "file:<f> not exist." and exits 0, core/io.hpp:27-30). */
int c2g_graph_load(const char* dir, int variant, int device, c2g_graph** out);

/* Build a graph from host CSR arrays (vlist[V+1], elist/wlist/flist[E]); wlist or
 * flist may be NULL.  Same device layout as c2g_graph_load. */
int c2g_graph_create(int device, int32_t V, int64_t E, const int32_t* vlist,
                     const int32_t* elist, const int32_t* wlist, const float* flist,
                     c2g_graph** out);

/* Attach pruned records (hvlist[R+1], helist/hwlist[hvlist[R]]).  hw_is_float selects
 * float (ppr/) or int32 (sssp/) weights.  record_vertex[R] (may be NULL) is the
 * record->vertex sidecar needed by C2G_SEEDS_EXACT. */
int c2g_graph_set_records(c2g_graph* g, int32_t R, const int32_t* hvlist,
                          const int32_t* helist, const void* hwlist, int hw_is_float,
                          const int32_t* record_vertex);

void c2g_graph_free(c2g_graph* g);
int  c2g_graph_info(const c2g_graph* g, int32_t* V, int64_t* E, int32_t* R);
/* Use the caller's CUDA stream (cudaStream_t passed as void*) instead of the handle's. */
int  c2g_graph_set_stream(c2g_graph* g, void* stream);
/* Watchdog of the persistent launches (no counterpart in the reference, whose software
 * grid barrier spins without limit, src/sssp/purn/Main.cu:173-189).  Every grid barrier
 * wait of a launch on this handle gives up after barrier_timeout_ms (0: the defaults,
 * 2 s single-query, 4 s batched); the call then returns C2G_ERR_TIMEOUT with
 * C2G_FLAG_BARRIER_TIMEOUT in the stats, and the handle stays usable.
 * stall_next_sssp = 1 makes the next c2g_sssp launch's barriers wait for one block more
 * than the grid has, so the wait runs out on purpose: a failure-detection test that
 * faults and hangs nothing. */
int  c2g_graph_set_watchdog(c2g_graph* g, int32_t barrier_timeout_ms, int32_t stall_next_sssp);
/* Tracing (no counterpart in the reference): time per phase of the last SSSP / PPR
 * launch on this handle, single or batched, as seen by block 0 at each grid barrier
 * (waits included): ms[0] initialisation, ms[1] frontier build / apply / far-pile
 * filter, ms[2] expansion / push, ms[3] reserved (0).  The phases add up to the
 * launch's device time. */
int  c2g_graph_last_phases(const c2g_graph* g, double ms[4]);
/* Tracing (no counterpart in the reference): per-round trace of the last batched launch
 * (c2g_sssp_batch / c2g_ppr_batch, or a session epoch) on this handle, up to 1024 rounds:
 * ms[i] the device time of round i (as block 0 sees it from one round's start to the
 * next), first_ms[i] the part of it up to the end of the round's first phase (PPR: the
 * push or pull, the apply sweep follows; SSSP: the expansion or pull, the next mask sweep
 * follows), work[i] its work units (PPR: (query, edge) pushes; SSSP: edge-word steps),
 * shape[i] 1 for a pull round, 0 otherwise.  Arrays hold `cap` entries (any may be NULL);
 * *n gets the number of rounds (0 when no batched launch finished cleanly). */
int  c2g_graph_last_rounds(c2g_graph* g, int32_t cap, double* ms, double* first_ms, int64_t* work, int32_t* shape,
                           int32_t* n);

/* ---- SSSP -------------------------------------------------------------------------- */
/* Source-skip rule of the drop-in programs: sssp-base skips sources without
 * out-edges (src/sssp/base/Main.cu:61-64); sssp-purn also skips sources whose record
 * holds more than 1000 seeds (src/sssp/purn/Main.cu:68-71).  pruned=0/1 selects the
 * rule; mode is a c2g_seed_mode. */
int c2g_sssp_resolve_source(const c2g_graph* g, int32_t source, int pruned, int mode,
                            int32_t* adjusted);

/* Single-source shortest paths with int32 weights; unreachable = 1999999999
 * (src/sssp/base/Main.cu:121).  Replaces CalcuSSSP (src/sssp/base/Main.cu:109-356,
 * src/sssp/purn/Main.cu:136-393) and its host loop.  use_seeds=0 runs the plain
 * traversal (sssp-base); use_seeds=1 applies the source's pruned records selected by
 * seed_mode (sssp-purn).  dist has V entries; dist_on_device=1 means a device
 * pointer. */
int c2g_sssp(c2g_graph* g, int32_t source, int use_seeds, int seed_mode, int32_t* dist,
             int dist_on_device, c2g_stats* stats);

/* Tuning knobs of the SSSP kernel: delta (bucket width of the near/far split,
 * <=0 = no split), tile (edges per warp tile, power of two in [32, 4096]),
 * max_iter (round cap, reference 1000). */
int c2g_sssp_set_config(c2g_graph* g, int32_t delta, int32_t tile, int32_t max_iter);

/* Allocation-free single-source SSSP (no counterpart in the reference).  For callers
 * that cannot let the library allocate device memory: a host whose device memory is
 * owned by another allocator, or a serving loop that must not call cudaMalloc/cudaFree
 * after start-up, since they may synchronise the device.  It runs the c2g_sssp kernel on
 * caller-owned device arrays:
 *   row  int32[V+1]                       CSR row pointer
 *   adj  E pairs of (int32 target, int32 weight), 8 bytes per edge
 *   dist int32[V]                          output, unreachable = 1999999999
 * Its scratch is one static device array of about 6.4 MB, held on every GPU that uses
 * it until the process exits.  It bounds the graph to C2G_NOALLOC_MAX_V vertices and
 * C2G_NOALLOC_MAX_E edges; larger inputs return C2G_ERR_RANGE.
 * The call allocates nothing: no cudaMalloc, no cudaFree, no allocating library call.
 * The first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) with that device current; make that first call before any
 * stream capture.  Every call shares the array, so calls that overlap on the GPU race:
 * serialise them (one stream, or host-side ordering).  Work runs on `stream`
 * (cudaStream_t, NULL for the legacy default stream) and the call returns when the
 * traversal has finished. */
#define C2G_NOALLOC_MAX_V 262144
#define C2G_NOALLOC_MAX_E 4194304
int c2g_sssp_noalloc(const int32_t* row, const void* adj, int32_t V, int64_t E, int32_t source,
                     int32_t* dist, void* stream, c2g_stats* stats);

/* Output layouts of the batched calls. */
#define C2G_LAYOUT_QUERY_MAJOR  0  /* out[q * V + v] */
#define C2G_LAYOUT_VERTEX_MAJOR 1  /* out[v * n + q] */

/* Batched multi-tenant SSSP: n sources in one persistent launch with per-query bitmask
 * frontiers (the reference runs one CalcuSSSP launch per source,
 * src/sssp/purn/Main.cu:67-99, or two on two streams in its PM mode,
 * src/sssp/purn-perk/Main.cu:87-246).  Each query's distances equal c2g_sssp's for the
 * same source, seeds and mode.  dist holds n*V entries in `layout`. */
int c2g_sssp_batch(c2g_graph* g, int32_t n, const int32_t* sources, int use_seeds, int seed_mode,
                   int32_t* dist, int dist_on_device, int layout, c2g_stats* stats);

/* Expansion tiles of the batched SSSP (c2g_sssp_batch; no counterpart in the reference,
 * whose launch geometry is fixed at compile time, core/Util.cuh:31-34).  Warps take tiles
 * of edge-word steps; a round with at least min_tiles_per_warp tiles of big_steps per
 * warp walks those, a smaller round tiles of 128 steps.  big_steps: power of two in
 * [128, 4096] (128: always small tiles); min_tiles_per_warp: power of two in [1, 1024].
 * Defaults 512 and 16.  Distances do not depend on the setting. */
int c2g_sssp_batch_set_tile(c2g_graph* g, int32_t big_steps, int32_t min_tiles_per_warp);
int c2g_sssp_batch_get_tile(const c2g_graph* g, int32_t* big_steps, int32_t* min_tiles_per_warp);

/* Round shape of the batched SSSP (c2g_sssp_batch and resident SSSP batches; no
 * counterpart in the reference): a round whose frontier makes more than frac * E * Q
 * (query, edge) relaxations (Q = query slots, a multiple of 32) pulls over the reverse
 * CSR with int32 weights (built on first use): each target takes the minimum over its
 * in-edges from sources that improved in the previous round.  frac < 0: expand (push)
 * only; 0: pull every round; default 0.3.  Distances do not depend on the setting. */
int c2g_sssp_batch_set_pull(c2g_graph* g, float frac);
int c2g_sssp_batch_get_pull(const c2g_graph* g, float* frac);

/* Autotuner of those tiles and of the round shape (no counterpart in the reference):
 * times 128-step tiles and big_steps {256, 512, 1024, 2048} x min_tiles_per_warp
 * {4, 16, 64} on this batch (one warm-up launch, then `reps` timed), then, at the fastest
 * tiles, pull fractions {expand only, 0.15, 0.3, 0.5, 0.75}; rejects any candidate whose
 * distances differ from the first's on the first 8 queries, applies the fastest tiles
 * and fraction, returns the tiles, and writes every timing as JSON to json_path (may be
 * NULL). */
int c2g_sssp_batch_autotune(c2g_graph* g, int32_t n, const int32_t* sources, int use_seeds, int seed_mode,
                            int32_t reps, const char* json_path, int32_t* best_big_steps,
                            int32_t* best_min_tiles);

/* Autotuner: time every (delta, tile) candidate of the SSSP kernel on the sample
 * sources (distances must agree across candidates), apply the fastest to the handle,
 * return it, and write every timing as JSON to json_path (may be NULL).  The reference's
 * launch geometry is fixed at compile time (core/Util.cuh:31-34). */
int c2g_sssp_autotune(c2g_graph* g, int32_t n, const int32_t* sources, int use_seeds, int seed_mode,
                      const char* json_path, int32_t* best_delta, int32_t* best_tile);

/* ---- PPR / adsorption push ------------------------------------------------------- */
/* Forward push.  Replaces calcuatePPR (src/ppr/base/Main.cu:122-395,
 * src/ppr/purn/Main.cu:149-428, src/adsorption/w-base/Main.cu:124-395) and the seed
 * assembly of src/ppr/purn/Main.cu:78-101.  pr and res have V entries (res may be
 * NULL); on_device=1 means device pointers. */
int c2g_ppr(c2g_graph* g, int32_t source, const c2g_ppr_params* params, float* pr,
            float* res, int on_device, c2g_stats* stats);

/* Batched forward push: n sources in one persistent launch with per-query bitmask
 * frontiers (the reference launches calcuatePPR once per source,
 * src/ppr/purn/Main.cu:78-117).  Each query follows c2g_ppr's BSP push with the same
 * parameters (seeded = 1 applies each source's records + kept out-edges); FP32 results
 * equal it within summation order.  pr (and res, which may be NULL) hold n*V floats in
 * `layout`. */
int c2g_ppr_batch(c2g_graph* g, int32_t n, const int32_t* sources, const c2g_ppr_params* params,
                  float* pr, float* res, int on_device, int layout, c2g_stats* stats);

/* Round shapes of the push kernel.  A round whose frontier has more than E / pull_div
 * out-edges pulls over the reverse CSR (built on first use) instead of pushing
 * (pull_div = 0, the default: never).  A push round whose frontier has more than
 * E / dense_div out-edges adds its messages without tracking first touches and applies
 * them in one sweep over all vertices (dense_div = 0: never; default 16).  Results are
 * the same BSP rounds either way. */
int c2g_ppr_set_config(c2g_graph* g, int32_t pull_div, int32_t dense_div);

/* Round shapes of the batched push (c2g_ppr_batch; no counterpart in the reference, which
 * runs one query per launch).  A round whose frontier makes more
 * than ratio * E (query, edge) pushes pulls over the reverse CSR (built on first use):
 * each target gathers its in-neighbours' pushed residuals and sums the messages as FP32
 * pairs (about 47 bits of relative precision) before they meet the FP64 residual.
 * ratio < 0: push only; 0: pull every round; default 8.  Pull rounds need finite weights
 * and rmax >= 1e-30.  Results are the same BSP rounds either way, within summation
 * order. */
int c2g_ppr_batch_set_pull(c2g_graph* g, float ratio);

/* Autotuner of that round shape (no counterpart in the reference): times ratios {push only, 1, 2, 4, 8, 16, 32} on this
 * batch (one warm-up launch, then `reps` timed), rejects any whose pr differs from the
 * push-only run by more than L1 1e-6 per query (first 8 queries), applies the fastest
 * and writes every timing as JSON to json_path (may be NULL). */
int c2g_ppr_batch_autotune(c2g_graph* g, int32_t n, const int32_t* sources, const c2g_ppr_params* params,
                           int32_t reps, const char* json_path, float* best_ratio);

/* Reference defaults: PPR (alpha 0.2, rmax 0.001/(V+1), cap 500), and the adsorption
 * program (alpha 0.2, r0 10, pr0 8, rmax 1/V, cap 2000). */
int c2g_ppr_default_params(const c2g_graph* g, int adsorption, c2g_ppr_params* out);

/* ---- PPR adjoint ------------------------------------------------------------------- */
/* Gradient of L = sum over targets t of pi_source(t) with respect to every float edge
 * weight (flist order), pi being the base-mode push of c2g_ppr with `params`
 * (alpha = teleport, as src/ppr/base/Main.cu:146-150).  dL/dw(u,v) =
 * (1-alpha) * pi(u) * lambda(v), lambda = (I - (1-alpha) P)^{-1} 1_T computed by a
 * transposed push on the reverse CSR with threshold rmax_backward (no counterpart in the
 * reference; the forward push it differentiates replaces calcuatePPR).  Repeated targets
 * count with their multiplicity.  grad has E entries; pi_out / lambda_out (V entries,
 * may be NULL) return the two vectors; loss (may be NULL) returns L. */
int c2g_ppr_adjoint(c2g_graph* g, int32_t source, const c2g_ppr_params* params, int32_t n_targets,
                    const int32_t* targets, float rmax_backward, float* grad, float* pi_out,
                    float* lambda_out, double* loss, int on_device, c2g_stats* stats);

/* Replace the float edge weights (E entries, flist order) in place. */
int c2g_graph_set_weights(c2g_graph* g, const float* flist, int on_device);

/* ---- adsorption label propagation --------------------------------------------------- */
/* Y_v <- p_inj(v) I_v + p_cont(v) sum_{u->v} w(u,v) Y_u over 16 labels (label l seeded
 * at seed_vertices[l]), from Y = I, for `iterations` Jacobi steps, FP32; p_abnd goes to
 * the unstored dummy label.  The reference's adsorption programs carry no labels
 * (src/adsorption/w-base/Main.cu:124-395 is the PPR push, served by c2g_ppr); this is
 * the labelled form of the serving configuration.  p_* have V entries; Y_out has V*16
 * floats (row v = labels of v). */
int c2g_adsorption(c2g_graph* g, int32_t n_labels, const int32_t* seed_vertices, const float* p_inj,
                   const float* p_cont, const float* p_abnd, int32_t iterations, float* Y_out,
                   int on_device, c2g_stats* stats);

/* ---- serving loop ------------------------------------------------------------------ */
/* Continuous-batching request loop with the graph and per-query state resident on the
 * device (replaces the reference's C^2graph-PM CPU/GPU migration loop,
 * src/sssp/purn-perk/Main.cu:87-246).  One worker per request kind, each on its own
 * stream; the three kinds run on the device concurrently.  SSSP and PPR requests run in a
 * resident batch (c2g_session) in epochs of epoch_rounds rounds: a request that arrives
 * while others run takes a free slot at the next epoch and completes as soon as its own
 * query finishes.  Slots are bounded by an HBM budget split between the kinds (state
 * bytes per query).  With preempt_rounds > 0, a waiting request may take the slot of the
 * running query with the most rounds (at least preempt_rounds), which is evicted into a
 * device snapshot and resumed first when a slot frees.  A request's result equals the
 * corresponding single call (c2g_sssp / c2g_ppr base mode / c2g_adsorption). */
#define C2G_REQ_SSSP       0
#define C2G_REQ_PPR        1
#define C2G_REQ_ADSORPTION 2

typedef struct c2g_server c2g_server;

typedef struct c2g_server_config {
    int32_t max_batch;        /* queries per batched launch, per kind (1..1024)        */
    int32_t ads_iterations;   /* adsorption iterations                                 */
    float   alpha, rmax;      /* PPR parameters (base mode)                            */
    int64_t hbm_budget_bytes; /* admission budget for per-query state, 0 = 80% of free */
    int32_t epoch_rounds;     /* rounds per epoch of the SSSP / PPR batches (0: 4)     */
    int32_t preempt_rounds;   /* evict queries past this many rounds when requests wait
                                 and no slot is free (0: never)                         */
} c2g_server_config;

typedef struct c2g_request {
    int32_t kind;             /* C2G_REQ_*                                              */
    int32_t source;           /* SSSP / PPR source                                      */
    const int32_t* seeds;     /* adsorption: 16 seed vertices (copied at submit)        */
    void* out;                /* host result buffer or NULL: int32[V] SSSP distances,
                                 float[V] PPR pagerank, float[V*16] adsorption labels   */
} c2g_request;

typedef struct c2g_server_stats {
    int64_t completed;
    int64_t batches[3];
    int64_t pending[3];
    int64_t admit_cap[3];     /* queries per batch allowed by the HBM budget            */
    int64_t max_batch;        /* most queries of one kind running at once so far       */
    double  p50_ms, p99_ms;   /* latency percentiles of completed requests              */
    double  queries_per_s;    /* completed / (last completion - first submit)           */
    int64_t evictions;        /* queries moved to a snapshot to free a slot             */
} c2g_server_stats;

/* g must carry int32 weights (SSSP) and float weights (PPR, adsorption); p_* (V
 * entries, host) are the adsorption probabilities (may be NULL without adsorption). */
int c2g_server_create(c2g_graph* g, const float* p_inj, const float* p_cont, const float* p_abnd,
                      const c2g_server_config* cfg, c2g_server** out);
int c2g_server_submit(c2g_server* s, const c2g_request* req, int64_t* ticket);
/* Block until the request finishes (timeout_s <= 0: no limit); status is its result
 * code, latency_ms its submit-to-completion time. */
int c2g_server_wait(c2g_server* s, int64_t ticket, double timeout_s, int* status, double* latency_ms);
int c2g_server_get_stats(c2g_server* s, c2g_server_stats* out);
/* Finish queued requests, stop the workers and release the server. */
int c2g_server_destroy(c2g_server* s);

/* ---- resident batches: slot-level continuous batching, snapshot / evict --------------- */
/* A session keeps `slots` queries of one kind (C2G_REQ_SSSP: plain SSSP on the graph's
 * int32 weights; C2G_REQ_PPR: base-mode push with `params`, seeded = 0) resident on the
 * device and runs them in epochs of a bounded number of rounds of the batched kernels.
 * Between epochs each query's state (SSSP: distances and next-round lanes; PPR: pr, res,
 * pushed residuals, frontier and dangling lanes) rests in the batch arrays, so a query
 * admitted while others run joins at the next epoch, and a running query can be evicted
 * into a device-resident snapshot and resumed later, in this or another session on the
 * same graph, continuing the same rounds.  Results equal c2g_sssp / c2g_ppr (base mode)
 * for the same source: SSSP bit-exact, PPR within summation order.  PPR round caps
 * (params->max_iter) are per query.  Replaces the reference's C^2graph-PM split of a query
 * between GPU iterations and a CPU thread over a pinned ring of per-query snapshots
 * (src/sssp/purn-perk/SSSP.h:13-29, src/sssp/purn-perk/Main.cu:87-246,
 * src/ppr/w-purn-perk/Main.cu:91-275): here the query stays on the device and only
 * yields its slot.  A session has its own stream and workspace; calls on one session are
 * serialised. */
typedef struct c2g_session c2g_session;
typedef struct c2g_snapshot c2g_snapshot;

int c2g_session_create(c2g_graph* g, int kind, int32_t slots, const c2g_ppr_params* params, c2g_session** out);
/* Take a free slot for `source`; the query starts at the next step.  C2G_ERR_OVERFLOW when
 * every slot is taken. */
int c2g_session_admit(c2g_session* s, int32_t source, int32_t* slot);
/* Apply admissions and resumptions, run one epoch of at most `rounds` rounds (fewer when a
 * PPR query would pass its cap, or when every query finishes), and report the slots whose
 * query finished: their ids go to finished[0 .. min(n, cap)), n to *n_finished.  A finished
 * slot keeps its result until c2g_session_read.  stats (may be NULL): the epoch's rounds,
 * pushes / relaxations and device time. */
int c2g_session_step(c2g_session* s, int32_t rounds, int32_t* finished, int32_t cap, int32_t* n_finished,
                     c2g_stats* stats);
/* Result of a finished slot (SSSP: int32 distances; PPR: float pr and, if res_out is not
 * NULL, float res; V entries each, host or device memory), then free the slot.  stats (may
 * be NULL): source, rounds run, status flags (C2G_FLAG_ITER_CAP if the cap stopped it). */
int c2g_session_read(c2g_session* s, int32_t slot, void* out, float* res_out, int on_device, c2g_stats* stats);
/* Move a running query out of its slot into a snapshot in device memory (the caller owns
 * it); the slot is free at once. */
int c2g_session_evict(c2g_session* s, int32_t slot, c2g_snapshot** out);
/* Continue a snapshot in a free slot from the next step; on success the session owns the
 * snapshot. */
int c2g_session_resume(c2g_session* s, c2g_snapshot* snap, int32_t* slot);
void c2g_snapshot_free(c2g_snapshot* snap);
/* Slot state (0 free, 1 running, 2 finished), its source and the rounds it has run. */
int c2g_session_slot(c2g_session* s, int32_t slot, int32_t* state, int32_t* source, int32_t* rounds);
void c2g_session_free(c2g_session* s);

/* ---- offline tools (host) ---------------------------------------------------------- */
/* Seeded R-MAT graph written as <dir>/origin/{vlist,elist,wlist,flist}.bin with
 * V = 2^scale, self-loops and duplicate edges removed, wlist uniform in [wmin,wmax],
 * flist = per-vertex normalised uniform(0,1).  Replaces utils/convert2binary.cpp's
 * text path (utils/convert2binary.cpp:82-137) for synthetic inputs. */
int c2g_rmat_write(const char* dir, int scale, int edge_factor, uint64_t seed,
                   int32_t wmin, int32_t wmax, double a, double b, double c);

/* The same graph generated on GPU `device` (endpoint draws, sort and dedup, weights on the
 * device; the files are byte-identical to c2g_rmat_write's).  Like c2g_rmat_write it
 * stands in for the reference's text converter (utils/convert2binary.cpp:10-114). */
int c2g_rmat_write_gpu(const char* dir, int scale, int edge_factor, uint64_t seed, int32_t wmin, int32_t wmax,
                       double a, double b, double c, int device);

/* Text edge list -> <dir>/origin/{vlist,elist,wlist,flist}.bin, the bytes the reference's
 * convert2binary writes (utils/convert2binary.cpp:10-137): lines "src dst:dst:...", self-loops
 * dropped, rows sorted and deduplicated, V = largest id + 1, weights rand() % 100 + 1 from
 * glibc's unseeded rand() and flist = w / row sum.  Where the reference would stop with an
 * uncaught exception (a destination stoi rejects) or index out of range (a negative id),
 * returns C2G_ERR_FORMAT and writes nothing; a missing file is C2G_ERR_IO.  The three
 * outputs (may be NULL) are the reference's printed "Max Vertex Number", "Vertex Number"
 * and "Edge Number". */
int c2g_convert_text(const char* text_path, const char* dir, int64_t* max_vertex, int64_t* vertices,
                     int64_t* edges);

/* C^2graph-P pruners.  Byte-identical outputs to purn-sssp (src/purn-sssp.cpp:61-352)
 * and purn-ppr (src/purn-ppr.cpp:63-344); purn-sssp additionally writes the
 * record->vertex sidecar <dir>/sssp/hvmap.bin. */
int c2g_prune_sssp(const char* dir);
int c2g_prune_ppr(const char* dir);
/* purn-ppr for another teleport probability: a folded edge carries (1 - alpha) instead
 * of the reference's baked 0.8 (src/purn-ppr.cpp:244), so a seeded push with that alpha
 * on the pruned graph follows the unpruned push.  alpha = 0.2 writes exactly what
 * c2g_prune_ppr writes (1 - 0.2 and 0.8 are the same double). */
int c2g_prune_ppr_alpha(const char* dir, double alpha);
/* purn-ppr on a GPU: the same visits as c2g_prune_ppr_alpha in rounds of a speculative
 * schedule (every unvisited vertex of a window plans its visit and reserves the rows it
 * reads and writes; the visits that no earlier planned visit conflicts with run in
 * parallel, one warp each), writing the same six files byte for byte.  Replaces the
 * sequential pass of purn-ppr (src/purn-ppr.cpp:146-283) on `device`.  *ms (may be NULL)
 * gets the kernel time, *rounds (may be NULL) the number of rounds, phase_ns[4] (may be
 * NULL) the kernel time spent in the rounds' four phases: plan, check, commit, copy (each
 * with the grid barrier that ends it).  Returns C2G_ERR_OVERFLOW when a device
 * row pool runs out (nothing is written). */
int c2g_prune_ppr_device(const char* dir, double alpha, int device, float* ms, int32_t* rounds,
                         int64_t* phase_ns);
/* purn-sssp on a GPU: the visits of c2g_prune_sssp (rounds k = 1..29 over the vertices in
 * id order, src/purn-sssp.cpp:139-294) in rounds of the same speculative schedule, writing
 * the same seven files (sssp/ with the record->vertex sidecar hvmap.bin) byte for byte.
 * ms, rounds and phase_ns as for c2g_prune_ppr_device. */
int c2g_prune_sssp_device(const char* dir, int device, float* ms, int32_t* rounds, int64_t* phase_ns);

#ifdef __cplusplus
}
#endif
#endif /* C2GRAPH_H */
