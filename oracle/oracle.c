/*
 * oracle.c - CPU oracle for the C^2graph traversal path.  TEST INFRASTRUCTURE ONLY:
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg load it as the
 * checker or as the timed CPU baseline.  The product library never calls it.
 *
 * Each function restates the reference algorithm it follows (file:line in the
 * reference project):
 *   orc_bellman_ford   src/sssp/base-perk/SSSP.cpp:88-119 (the reference's own CPU
 *                      Bellman-Ford, the exact copy; not the purn-perk one)
 *   orc_dijkstra       independent exact check: shortest distances are unique, so any
 *                      exact method pins CalcuSSSP's fixed point
 *                      (src/sssp/base/Main.cu:109-356, src/sssp/purn/Main.cu:136-393)
 *   orc_sssp_seeded    the sssp-purn launch semantics: dis[source]=0, seeds by
 *                      atomicMin, frontier = seeds + source (src/sssp/purn/Main.cu:72-90,
 *                      160-181), then relaxation to the fixed point
 *   orc_ppr_push_{f64,f32}
 *                      BSP forward push of calcuatePPR (src/ppr/base/Main.cu:146-150,
 *                      src/ppr/purn/Main.cu:156-198 init/seeds, :248-360 push,
 *                      :379-407 frontier rule) in double or float
 *   orc_batch          one independent query per host thread, with or without each
 *                      query's first-hop seeds (CPU baseline, parallel checks)
 *   orc_sssp_certificate
 *                      size-independent exactness check of a distance vector: the
 *                      Bellman conditions of the fixed point CalcuSSSP computes
 *
 * Parity is pinned by tests/test_oracle_golden.py against fixtures made by the
 * reference's own code built from source (oracle/build.py, tests/golden/).
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_INF 1999999999 /* src/sssp/base/Main.cu:121 */

/* ---- SSSP -------------------------------------------------------------------------- */

/* Frontier Bellman-Ford over an existing distance vector, restating the reference CPU
 * routine: every frontier vertex relaxes all out-edges with the live distances; a
 * vertex joins the next frontier the first time it improves in a round.  Returns the
 * number of rounds. */
int orc_bellman_ford(int32_t V, const int32_t* row, const int32_t* col, const int32_t* w,
                     int32_t* dist, const int32_t* frontier, int32_t n_frontier) {
    if (n_frontier <= 0) return 0;
    int32_t* cur = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V > n_frontier ? V : n_frontier));
    int32_t* nxt = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V > 0 ? V : 1));
    char* flag = (char*)calloc((size_t)(V > 0 ? V : 1), 1);
    int32_t ncur = n_frontier, nnxt = 0, rounds = 0;
    memcpy(cur, frontier, sizeof(int32_t) * (size_t)n_frontier);
    while (ncur > 0) {
        ++rounds;
        nnxt = 0;
        for (int32_t a = 0; a < ncur; ++a) {
            const int32_t u = cur[a];
            if (row[u + 1] - row[u] <= 0) continue;
            for (int32_t j = row[u]; j < row[u + 1]; ++j) {
                const int32_t v = col[j];
                const int32_t nd = dist[u] + w[j];
                if (!flag[v] && dist[v] > nd) {
                    nxt[nnxt++] = v;
                    flag[v] = 1;
                }
                if (nd < dist[v]) dist[v] = nd;
            }
        }
        for (int32_t a = 0; a < nnxt; ++a) flag[nxt[a]] = 0;
        int32_t* t = cur;
        cur = nxt;
        nxt = t;
        ncur = nnxt;
    }
    free(cur);
    free(nxt);
    free(flag);
    return rounds;
}

/* binary min-heap of (dist, vertex) */
typedef struct { int32_t d, v; } hitem;

static void heap_push(hitem* h, int64_t* n, hitem x) {
    int64_t i = (*n)++;
    while (i > 0) {
        int64_t p = (i - 1) / 2;
        if (h[p].d <= x.d) break;
        h[i] = h[p];
        i = p;
    }
    h[i] = x;
}

static hitem heap_pop(hitem* h, int64_t* n) {
    hitem top = h[0], x = h[--(*n)];
    int64_t i = 0;
    for (;;) {
        int64_t c = 2 * i + 1;
        if (c >= *n) break;
        if (c + 1 < *n && h[c + 1].d < h[c].d) ++c;
        if (h[c].d >= x.d) break;
        h[i] = h[c];
        i = c;
    }
    if (*n > 0) h[i] = x;
    return top;
}

/* Multi-source Dijkstra: dist = min over (init_v[k], init_d[k]) of init_d + path. */
void orc_dijkstra(int32_t V, const int32_t* row, const int32_t* col, const int32_t* w,
                  int32_t n_init, const int32_t* init_v, const int32_t* init_d, int32_t* dist) {
    for (int32_t v = 0; v < V; ++v) dist[v] = ORC_INF;
    int64_t cap = (int64_t)row[V] + n_init + 1, n = 0;
    hitem* h = (hitem*)malloc(sizeof(hitem) * (size_t)cap);
    for (int32_t k = 0; k < n_init; ++k) {
        if (init_d[k] < dist[init_v[k]]) {
            dist[init_v[k]] = init_d[k];
            hitem it = {init_d[k], init_v[k]};
            heap_push(h, &n, it);
        }
    }
    while (n > 0) {
        hitem t = heap_pop(h, &n);
        if (t.d != dist[t.v]) continue;
        for (int32_t j = row[t.v]; j < row[t.v + 1]; ++j) {
            const int32_t v = col[j];
            const int32_t nd = t.d + w[j];
            if (nd < dist[v]) {
                dist[v] = nd;
                hitem it = {nd, v};
                heap_push(h, &n, it);
            }
        }
    }
    free(h);
}

/* sssp-base / sssp-purn launch semantics: dis = INF; dis[source] = 0; each seed
 * (seed_v[k], seed_w[k]) lowers dis[seed_v[k]] to seed_w[k]; frontier = seeds then the
 * source; relax to the fixed point with the reference CPU Bellman-Ford.  Returns the
 * number of rounds. */
int orc_sssp_seeded(int32_t V, const int32_t* row, const int32_t* col, const int32_t* w,
                    int32_t source, int32_t n_seeds, const int32_t* seed_v, const int32_t* seed_w,
                    int32_t* dist) {
    for (int32_t v = 0; v < V; ++v) dist[v] = ORC_INF;
    dist[source] = 0;
    for (int32_t k = 0; k < n_seeds; ++k)
        if (seed_w[k] < dist[seed_v[k]]) dist[seed_v[k]] = seed_w[k];
    int32_t* fr = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n_seeds + 1));
    for (int32_t k = 0; k < n_seeds; ++k) fr[k] = seed_v[k];
    fr[n_seeds] = source;
    int r = orc_bellman_ford(V, row, col, w, dist, fr, n_seeds + 1);
    free(fr);
    return r;
}

/* Optimality certificate of a distance vector for sources S (dist 0) and seeds (v, w):
 *   (a) dist[s] = 0 for s in S, dist[v] <= w for each seed;
 *   (b) no edge improves a distance: dist[v] <= dist[u] + w(u,v) whenever dist[u] is finite;
 *   (c) every other finite dist[v] is achieved by a tight in-edge (dist[u] + w(u,v) ==
 *       dist[v]) or by a seed (w == dist[v]);
 *   (d) unreachable vertices hold exactly ORC_INF.
 * With positive weights (a)-(c) pin dist to the shortest distances (tight in-edges lead
 * back, strictly decreasing, to a source or seed; no edge shortens any of them), so the
 * check replaces an oracle run on graphs too large for one.  Returns the number of
 * violating vertices (0: certified); bad_vertex gets the first one. */
int64_t orc_sssp_certificate(int32_t V, const int32_t* row, const int32_t* col, const int32_t* w,
                             int32_t n_src, const int32_t* src, int32_t n_seeds, const int32_t* seed_v,
                             const int32_t* seed_w, const int32_t* dist, int32_t* bad_vertex) {
    char* tight = (char*)calloc((size_t)(V > 0 ? V : 1), 1);
    int64_t bad = 0;
    *bad_vertex = -1;
#define ORC_BAD(v)                              \
    do {                                        \
        if (*bad_vertex < 0) *bad_vertex = (v); \
        ++bad;                                  \
    } while (0)
    for (int32_t k = 0; k < n_src; ++k) {
        if (dist[src[k]] != 0) ORC_BAD(src[k]);
        tight[src[k]] = 1;
    }
    for (int32_t k = 0; k < n_seeds; ++k) {
        if (dist[seed_v[k]] > seed_w[k]) ORC_BAD(seed_v[k]);
        if (dist[seed_v[k]] == seed_w[k]) tight[seed_v[k]] = 1;
    }
    for (int32_t u = 0; u < V; ++u) {
        const int32_t du = dist[u];
        if (du < 0 || du > ORC_INF) ORC_BAD(u);
        if (du >= ORC_INF) continue;
        for (int32_t j = row[u]; j < row[u + 1]; ++j) {
            const int64_t nd = (int64_t)du + w[j];
            const int32_t v = col[j];
            if ((int64_t)dist[v] > nd) ORC_BAD(v);
            if ((int64_t)dist[v] == nd) tight[v] = 1;
        }
    }
    for (int32_t v = 0; v < V; ++v)
        if (dist[v] < ORC_INF && !tight[v]) ORC_BAD(v);
#undef ORC_BAD
    free(tight);
    return bad;
}

/* ---- PPR forward push -------------------------------------------------------------- */

/* BSP forward push.  Round: every frontier vertex u pops r = res[u] (res[u] = 0) and
 * sends (1-alpha)*r*w to each out-neighbour's message; then every vertex that got a
 * message adds it to its residual and, if residual > rmax, gains alpha*residual in pr
 * and joins the next frontier.  Init (seeded = 0): pr[s] = pr0, frontier {s} with
 * residual r0.  Init (seeded = 1): pr[s] = alpha; every seed (v, w) adds
 * (1-alpha)*alpha*w to pr[v] and (1-alpha)*w to res[v]; the distinct seed vertices form
 * the first frontier.  degree_scaled = 1 switches the activation test to
 * residual > outdeg*rmax, the rule of the reference's CPU forward_push
 * (src/ppr/w-purn-perk/PPR.cpp:220), which pins this restatement against that code.
 * Returns the number of rounds; counters (may be NULL) get [popped, edges, touched]. */
#define ORC_PPR_BODY(T)                                                                    \
    for (int32_t v = 0; v < V; ++v) { pr[v] = 0; res[v] = 0; }                             \
    T* msg = (T*)calloc((size_t)(V > 0 ? V : 1), sizeof(T));                               \
    char* act = (char*)calloc((size_t)(V > 0 ? V : 1), 1);                                 \
    char* inq = (char*)calloc((size_t)(V > 0 ? V : 1), 1);                                 \
    int32_t* cur = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V > 0 ? V : 1));            \
    int32_t* nxt = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V > 0 ? V : 1));            \
    int32_t* touched = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V > 0 ? V : 1));        \
    int32_t ncur = 0;                                                                      \
    const T a = (T)alpha, one_m_a = (T)1 - (T)alpha;                                       \
    int64_t c_pop = 0, c_edges = 0, c_touch = 0;                                           \
    if (!seeded) {                                                                         \
        res[source] = (T)r0;                                                               \
        pr[source] += (T)pr0;                                                              \
        cur[ncur++] = source;                                                              \
    } else {                                                                               \
        res[source] = 0;                                                                   \
        pr[source] = a;                                                                    \
        for (int32_t k = 0; k < n_seeds; ++k) {                                            \
            pr[seed_v[k]] += one_m_a * a * (T)seed_w[k];                                   \
            res[seed_v[k]] += one_m_a * (T)seed_w[k];                                      \
        }                                                                                  \
        for (int32_t k = 0; k < n_seeds; ++k)                                              \
            if (!inq[seed_v[k]]) { inq[seed_v[k]] = 1; cur[ncur++] = seed_v[k]; }          \
        for (int32_t k = 0; k < ncur; ++k) inq[cur[k]] = 0;                                \
    }                                                                                      \
    int32_t rounds = 0;                                                                    \
    while (ncur > 0 && rounds < max_iter) {                                                \
        ++rounds;                                                                          \
        int32_t ntouch = 0;                                                                \
        c_pop += ncur;                                                                     \
        for (int32_t k = 0; k < ncur; ++k) {                                               \
            const int32_t u = cur[k];                                                      \
            const T ru = res[u];                                                           \
            res[u] = 0;                                                                    \
            const T q = one_m_a * ru;                                                      \
            c_edges += row[u + 1] - row[u];                                                \
            for (int32_t j = row[u]; j < row[u + 1]; ++j) {                                \
                const int32_t v = col[j];                                                  \
                msg[v] += q * (T)f[j];                                                     \
                if (!act[v]) { act[v] = 1; touched[ntouch++] = v; }                        \
            }                                                                              \
        }                                                                                  \
        c_touch += ntouch;                                                                 \
        int32_t nn = 0;                                                                    \
        for (int32_t k = 0; k < ntouch; ++k) {                                             \
            const int32_t v = touched[k];                                                  \
            act[v] = 0;                                                                    \
            res[v] += msg[v];                                                              \
            msg[v] = 0;                                                                    \
            const T thr = degree_scaled ? (T)(row[v + 1] - row[v]) * (T)rmax : (T)rmax;   \
            if (res[v] > thr) {                                                            \
                pr[v] += a * res[v];                                                       \
                nxt[nn++] = v;                                                             \
            }                                                                              \
        }                                                                                  \
        int32_t* t = cur; cur = nxt; nxt = t; ncur = nn;                                   \
    }                                                                                      \
    if (counters) { counters[0] = c_pop; counters[1] = c_edges; counters[2] = c_touch; }   \
    free(msg); free(act); free(inq); free(cur); free(nxt); free(touched);                  \
    return rounds;

int orc_ppr_push_f64(int32_t V, const int32_t* row, const int32_t* col, const float* f,
                     int32_t source, double alpha, double rmax, double r0, double pr0,
                     int32_t max_iter, int32_t seeded, int32_t degree_scaled, int32_t n_seeds,
                     const int32_t* seed_v, const float* seed_w, double* pr, double* res,
                     int64_t* counters) {
    ORC_PPR_BODY(double)
}

int orc_ppr_push_f32(int32_t V, const int32_t* row, const int32_t* col, const float* f,
                     int32_t source, double alpha, double rmax, double r0, double pr0,
                     int32_t max_iter, int32_t seeded, int32_t degree_scaled, int32_t n_seeds,
                     const int32_t* seed_v, const float* seed_w, float* pr, float* res,
                     int64_t* counters) {
    ORC_PPR_BODY(float)
}

/* ---- batched queries: one query per thread (CPU baseline and parallel checks) ------- */

typedef struct {
    int kind; /* 0 sssp (reference CPU Bellman-Ford from the source and its seeds),
                 1 ppr BSP push in float, 2 the same push in double */
    int32_t V;
    const int32_t *row, *col, *w;
    const float* f;
    const int32_t* sources;
    const int32_t* seed_off; /* NULL: no seeds; else seeds of query q in [seed_off[q], seed_off[q+1]) */
    const int32_t* seed_v;
    const void* seed_w; /* int32 (sssp) or float (ppr) */
    int32_t nq;
    int32_t* next; /* shared work counter */
    pthread_mutex_t* mu;
    double alpha, rmax;
    int32_t max_iter;
    int64_t edges;     /* per-thread edges relaxed */
    int32_t* dist_out; /* optional: nq*V */
    float* pr_out;     /* optional: nq*V (kind 1) */
    double* pr64_out;  /* optional: nq*V (kind 2) */
    double* res64_out; /* optional: nq*V (kind 2) */
} orc_worker;

static void* orc_worker_main(void* p) {
    orc_worker* wk = (orc_worker*)p;
    int32_t V = wk->V;
    const size_t nv = (size_t)(V > 0 ? V : 1);
    int32_t* dist = (int32_t*)malloc(sizeof(int32_t) * nv);
    float* pr = (float*)malloc(sizeof(float) * nv);
    float* res = (float*)malloc(sizeof(float) * nv);
    double* pr64 = wk->kind == 2 ? (double*)malloc(sizeof(double) * nv) : NULL;
    double* res64 = wk->kind == 2 ? (double*)malloc(sizeof(double) * nv) : NULL;
    for (;;) {
        pthread_mutex_lock(wk->mu);
        int32_t q = (*wk->next)++;
        pthread_mutex_unlock(wk->mu);
        if (q >= wk->nq) break;
        const int32_t s = wk->sources[q];
        int32_t ns = 0;
        const int32_t* sv = NULL;
        const void* sw = NULL;
        if (wk->seed_off) {
            ns = wk->seed_off[q + 1] - wk->seed_off[q];
            sv = wk->seed_v + wk->seed_off[q];
            sw = wk->kind == 0 ? (const void*)((const int32_t*)wk->seed_w + wk->seed_off[q])
                               : (const void*)((const float*)wk->seed_w + wk->seed_off[q]);
        }
        if (wk->kind == 0) {
            orc_sssp_seeded(V, wk->row, wk->col, wk->w, s, ns, sv, (const int32_t*)sw, dist);
            for (int32_t v = 0; v < V; ++v)
                if (dist[v] != ORC_INF) wk->edges += wk->row[v + 1] - wk->row[v];
            if (wk->dist_out) memcpy(wk->dist_out + (size_t)q * V, dist, sizeof(int32_t) * (size_t)V);
        } else if (wk->kind == 1) {
            int64_t c[3];
            orc_ppr_push_f32(V, wk->row, wk->col, wk->f, s, wk->alpha, wk->rmax, 1.0, wk->alpha, wk->max_iter,
                             wk->seed_off != NULL, 0, ns, sv, (const float*)sw, pr, res, c);
            wk->edges += c[1];
            if (wk->pr_out) memcpy(wk->pr_out + (size_t)q * V, pr, sizeof(float) * (size_t)V);
        } else {
            int64_t c[3];
            orc_ppr_push_f64(V, wk->row, wk->col, wk->f, s, wk->alpha, wk->rmax, 1.0, wk->alpha, wk->max_iter,
                             wk->seed_off != NULL, 0, ns, sv, (const float*)sw, pr64, res64, c);
            wk->edges += c[1];
            if (wk->pr64_out) memcpy(wk->pr64_out + (size_t)q * V, pr64, sizeof(double) * (size_t)V);
            if (wk->res64_out) memcpy(wk->res64_out + (size_t)q * V, res64, sizeof(double) * (size_t)V);
        }
    }
    free(dist);
    free(pr);
    free(res);
    free(pr64);
    free(res64);
    return NULL;
}

/* Run nq independent queries on nthreads host threads.  kind 0: SSSP (edges = out-edges
 * of reached vertices); kind 1: PPR push in float, kind 2: in double (edges = edges
 * pushed).  With seed_off, query q applies its seeds: the sssp-purn first hop
 * (src/sssp/purn/Main.cu:72-90) or the ppr-purn one (src/ppr/purn/Main.cu:78-101) with
 * the push's base values (pr0 = alpha, r0 = 1) unused.  Returns the total edge count. */
int64_t orc_batch(int kind, int32_t V, const int32_t* row, const int32_t* col, const int32_t* w,
                  const float* f, int32_t nq, const int32_t* sources, const int32_t* seed_off,
                  const int32_t* seed_v, const void* seed_w, double alpha, double rmax, int32_t max_iter,
                  int32_t nthreads, int32_t* dist_out, float* pr_out, double* pr64_out, double* res64_out) {
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
    orc_worker* wk = (orc_worker*)calloc((size_t)nthreads, sizeof(orc_worker));
    pthread_mutex_t mu;
    pthread_mutex_init(&mu, NULL);
    int32_t next = 0;
    for (int t = 0; t < nthreads; ++t) {
        orc_worker x = {kind, V, row, col, w, f, sources, seed_off, seed_v, seed_w, nq, &next, &mu, alpha, rmax,
                        max_iter, 0, dist_out, pr_out, pr64_out, res64_out};
        wk[t] = x;
        pthread_create(&th[t], NULL, orc_worker_main, &wk[t]);
    }
    int64_t edges = 0;
    for (int t = 0; t < nthreads; ++t) {
        pthread_join(th[t], NULL);
        edges += wk[t].edges;
    }
    pthread_mutex_destroy(&mu);
    free(th);
    free(wk);
    return edges;
}
