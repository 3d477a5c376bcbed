/*
 * ingest.c - CPU oracle for the inputs of the traversal path: the seeded R-MAT writer
 * and the C^2graph-P pruners.  TEST INFRASTRUCTURE ONLY: tests/ pin these functions
 * against the golden fixtures, and bench.py's reference arm and CPU-baseline leg use
 * them to build their inputs without loading the product library.
 *
 *   orc_rmat_write     the synthetic input in the reference's origin/ layout
 *                      (vlist int32[V+1], elist int32[E], wlist int32[E], flist
 *                      float32[E], the layout utils/convert2binary.cpp:98-129 writes).
 *                      R-MAT recursive quadrant choice (Chakrabarti, Zhan, Faloutsos,
 *                      SDM 2004) with counter-based splitmix64 draws (Steele, Lea,
 *                      Flood, OOPSLA 2014) keyed by (seed, stream, index): stream 1 the
 *                      endpoints (one 64-bit draw per two levels, low half first),
 *                      stream 2 the int32 weights (uniform by modulo over the range),
 *                      stream 3 the flist values (24 random bits + 0.5, over 2^24),
 *                      normalised per row by their double sum in row order.  Rows are
 *                      sorted by target, self-loops and duplicates removed.
 *   orc_prune_sssp     purn-sssp (src/purn-sssp.cpp:61-352): rounds k = 0..29 over all
 *                      vertices in id order (:139-150); a vertex with live in-degree in
 *                      [1, 29] and out-edges is pruned once (:151-286); int weights,
 *                      min-combination (:250-272), folded edges that would point back at
 *                      their root are skipped (:244,263).  Also writes the record->vertex
 *                      sidecar sssp/hvmap.bin (pruning order), which the reference does
 *                      not write.
 *   orc_prune_ppr      purn-ppr (src/purn-ppr.cpp:63-344): one pass in id order with
 *                      in-degree bound 5 (:146-152); every vertex gets a record, empty
 *                      when not pruned (:281-283); float weights combined as
 *                      (w * keep) * w' in double and rounded to float (:244-259), keep =
 *                      0.8 in the reference.
 *
 *   orc_prune_depth    either pruner with a dependency analysis of its visiting order
 *                      (not a restatement: an analysis of the sequential algorithm, for
 *                      the question whether a parallel pruner could reproduce its bytes).
 *   orc_prune_speculative, orc_prune_ppr_speculative
 *                      either pruner's steps in rounds of the reservation-based parallel
 *                      schedule the device pruners run, on the CPU, to check that schedule
 *                      against the sequential pass's bytes.
 *
 * The pruners keep the reference's per-vertex state: the out-rows as sorted
 * (target, weight) lists built from each row's distinct pairs without self-loops
 * (core/util.hpp:80-96), the in-rows as sorted (source, alive) lists
 * (src/purn-sssp.cpp:39-58), and the live in-degrees.  The reference advances a cursor
 * per root with a linear walk (src/purn-sssp.cpp:198-200); a binary search over the
 * same range lands on the same position (the walk stops at the first index at or past
 * the cursor whose target is >= v, or at the row's last index).
 */
#include <errno.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

/* ---- files ---------------------------------------------------------------------------- */

static int orc_mkdir(const char* p) {
    if (mkdir(p, 0755) == 0 || errno == EEXIST) return 0;
    return -2;
}

static int orc_write4(const char* dir, const char* sub, const char* name, const void* a, size_t n) {
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s/%s.bin", dir, sub, name);
    FILE* f = fopen(path, "wb");
    if (!f) return -2;
    size_t w = n ? fwrite(a, 4, n, f) : 0;
    int rc = fclose(f);
    return (w != n || rc != 0) ? -2 : 0;
}

static int32_t* orc_read4(const char* dir, const char* sub, const char* name, size_t* n) {
    char path[4096];
    snprintf(path, sizeof(path), "%s/%s/%s.bin", dir, sub, name);
    FILE* f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long bytes = ftell(f);
    fseek(f, 0, SEEK_SET);
    *n = (size_t)bytes / 4;
    int32_t* a = (int32_t*)malloc(*n ? *n * 4 : 4);
    if (*n && fread(a, 4, *n, f) != *n) {
        free(a);
        a = NULL;
    }
    fclose(f);
    return a;
}

/* ---- R-MAT ------------------------------------------------------------------------------ */

static uint64_t orc_splitmix(uint64_t x) {
    x += 0x9e3779b97f4a7c15ULL;
    x = (x ^ (x >> 30)) * 0xbf58476d1ce4e5b9ULL;
    x = (x ^ (x >> 27)) * 0x94d049bb133111ebULL;
    return x ^ (x >> 31);
}

/* draw k of item `index` in `stream` */
static uint64_t orc_draw(uint64_t seed, uint64_t stream, uint64_t index, uint64_t k) {
    const uint64_t key = orc_splitmix(seed ^ (stream * 0xd1342543de82ef95ULL));
    return orc_splitmix(key + index * 0x9e3779b97f4a7c15ULL + k);
}

static int orc_cmp_i32(const void* a, const void* b) {
    const int32_t x = *(const int32_t*)a, y = *(const int32_t*)b;
    return (x > y) - (x < y);
}

int orc_rmat_write(const char* dir, int scale, int edge_factor, uint64_t seed, int32_t wmin, int32_t wmax,
                   double a, double b, double c) {
    if (!dir || scale < 1 || scale > 30 || edge_factor < 1 || wmin > wmax) return -1;
    const int64_t V = (int64_t)1 << scale;
    const int64_t M = (int64_t)edge_factor * V;
    if (M >= ((int64_t)1 << 31)) return -1;
    /* cumulative quadrant thresholds over 32-bit draws: a, a+b, a+b+c */
    const double two32 = 4294967296.0;
    const uint64_t t1 = (uint64_t)floor(a * two32);
    const uint64_t t2 = t1 + (uint64_t)floor(b * two32);
    const uint64_t t3 = t2 + (uint64_t)floor(c * two32);
    int32_t* src = (int32_t*)malloc(sizeof(int32_t) * (size_t)M);
    int32_t* dst = (int32_t*)malloc(sizeof(int32_t) * (size_t)M);
    int64_t* start = (int64_t*)calloc((size_t)V + 1, sizeof(int64_t));
    if (!src || !dst || !start) return -5;
    for (int64_t i = 0; i < M; ++i) {
        uint64_t s = 0, d = 0, r = 0;
        for (int l = 0; l < scale; ++l) {
            if (!(l & 1)) r = orc_draw(seed, 1, (uint64_t)i, (uint64_t)(l / 2));
            const uint64_t q = (l & 1) ? (r >> 32) : (r & 0xffffffffULL);
            const uint64_t bit = (uint64_t)1 << (scale - 1 - l);
            if (q >= t3) {
                s |= bit;
                d |= bit;
            } else if (q >= t2) {
                s |= bit;
            } else if (q >= t1) {
                d |= bit;
            }
        }
        src[i] = (int32_t)s;
        dst[i] = (int32_t)d;
        if (s != d) start[s + 1]++;
    }
    for (int64_t v = 0; v < V; ++v) start[v + 1] += start[v];
    int32_t* tg = (int32_t*)malloc(sizeof(int32_t) * (size_t)(start[V] ? start[V] : 1));
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)V);
    memcpy(fill, start, sizeof(int64_t) * (size_t)V);
    for (int64_t i = 0; i < M; ++i)
        if (src[i] != dst[i]) tg[fill[src[i]]++] = dst[i];
    free(src);
    free(dst);
    free(fill);
    int32_t* vl = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V + 1));
    vl[0] = 0;
    int64_t E = 0;
    for (int64_t v = 0; v < V; ++v) {
        int32_t* row = tg + start[v];
        const int64_t n = start[v + 1] - start[v];
        qsort(row, (size_t)n, sizeof(int32_t), orc_cmp_i32);
        for (int64_t k = 0; k < n; ++k)
            if (k == 0 || row[k] != row[k - 1]) tg[E++] = row[k]; /* compacts in place: E <= start[v] + k */
        vl[v + 1] = (int32_t)E;
    }
    free(start);
    int32_t* wl = (int32_t*)malloc(sizeof(int32_t) * (size_t)(E ? E : 1));
    float* fl = (float*)malloc(sizeof(float) * (size_t)(E ? E : 1));
    const uint64_t range = (uint64_t)((int64_t)wmax - (int64_t)wmin + 1);
    for (int64_t v = 0; v < V; ++v) {
        double sum = 0.0;
        for (int64_t e = vl[v]; e < vl[v + 1]; ++e) {
            wl[e] = (int32_t)((int64_t)wmin + (int64_t)(orc_draw(seed, 2, (uint64_t)e, 0) % range));
            const float u = (float)(((double)(orc_draw(seed, 3, (uint64_t)e, 0) >> 40) + 0.5) / 16777216.0);
            fl[e] = u;
            sum += (double)u;
        }
        for (int64_t e = vl[v]; e < vl[v + 1]; ++e) fl[e] = (float)((double)fl[e] / sum);
    }
    char p[4096];
    int rc = orc_mkdir(dir);
    const char* subs[3] = {"origin", "sssp", "ppr"};
    for (int k = 0; k < 3 && !rc; ++k) {
        snprintf(p, sizeof(p), "%s/%s", dir, subs[k]);
        rc = orc_mkdir(p);
    }
    if (!rc) rc = orc_write4(dir, "origin", "vlist", vl, (size_t)V + 1);
    if (!rc) rc = orc_write4(dir, "origin", "elist", tg, (size_t)E);
    if (!rc) rc = orc_write4(dir, "origin", "wlist", wl, (size_t)E);
    if (!rc) rc = orc_write4(dir, "origin", "flist", fl, (size_t)E);
    free(vl);
    free(tg);
    free(wl);
    free(fl);
    return rc;
}

/* ---- pruners ---------------------------------------------------------------------------- */

typedef struct { /* out-row: sorted targets with their 32-bit weights (int or float bits) */
    int32_t n, cap;
    int32_t* t;
    uint32_t* w;
} orow;

typedef struct { /* in-row: sorted sources with an alive flag */
    int32_t n, cap;
    int32_t* s;
    unsigned char* alive;
} irow;

typedef struct { /* growable int32 list */
    int64_t n, cap;
    uint32_t* a;
} ilist;

static void il_push(ilist* l, uint32_t x) {
    if (l->n == l->cap) {
        l->cap = l->cap ? 2 * l->cap : 64;
        l->a = (uint32_t*)realloc(l->a, sizeof(uint32_t) * (size_t)l->cap);
    }
    l->a[l->n++] = x;
}

/* first index in t[lo, hi) with t[idx] >= key, or hi */
static int32_t lower_i32(const int32_t* t, int32_t lo, int32_t hi, int32_t key) {
    while (lo < hi) {
        const int32_t mid = lo + (hi - lo) / 2;
        if (t[mid] < key)
            lo = mid + 1;
        else
            hi = mid;
    }
    return lo;
}

static uint32_t f2u(float f) {
    uint32_t u;
    memcpy(&u, &f, 4);
    return u;
}
static float u2f(uint32_t u) {
    float f;
    memcpy(&f, &u, 4);
    return f;
}

typedef struct {
    int ppr;     /* 0: purn-sssp rules, 1: purn-ppr rules */
    double keep; /* purn-ppr factor of a folded edge */
} prune_rule;

/* weight of a folded edge i->v seen from root k: d3 = w(i,v), dk = w(root,i) */
static uint32_t fold_new(const prune_rule* r, uint32_t d3, uint32_t dk) {
    if (!r->ppr) return (uint32_t)((int32_t)d3 + (int32_t)dk);
    return f2u((float)((double)u2f(d3) * r->keep * (double)u2f(dk)));
}
static uint32_t fold_hit(const prune_rule* r, uint32_t old, uint32_t d3, uint32_t dk) {
    if (!r->ppr) {
        const int32_t nw = (int32_t)d3 + (int32_t)dk;
        return (int32_t)old < nw ? old : (uint32_t)nw;
    }
    return f2u((float)((double)u2f(old) + (double)u2f(d3) * r->keep * (double)u2f(dk)));
}

typedef struct {
    int32_t t;
    uint32_t w;
} tw_pair;

static int cmp_pair_int(const void* a, const void* b) {
    const tw_pair *x = (const tw_pair*)a, *y = (const tw_pair*)b;
    if (x->t != y->t) return (x->t > y->t) - (x->t < y->t);
    return ((int32_t)x->w > (int32_t)y->w) - ((int32_t)x->w < (int32_t)y->w);
}

static int cmp_pair_float(const void* a, const void* b) {
    const tw_pair *x = (const tw_pair*)a, *y = (const tw_pair*)b;
    if (x->t != y->t) return (x->t > y->t) - (x->t < y->t);
    return (u2f(x->w) > u2f(y->w)) - (u2f(x->w) < u2f(y->w));
}

/* Rows from a CSR: distinct (target, weight) pairs without self-loops, sorted (the
 * reference inserts them into a std::set, core/util.hpp:80-96), and the in-rows of the
 * distinct targets (src/purn-sssp.cpp:39-58). */
static void prune_rows(int32_t V, const int32_t* vl, const int32_t* el, const uint32_t* wl, int ppr, orow* out,
                       irow* in, int32_t* indeg) {
    int32_t* icnt = (int32_t*)calloc((size_t)(V ? V : 1), sizeof(int32_t));
    int32_t maxdeg = 1;
    for (int32_t v = 0; v < V; ++v)
        if (vl[v + 1] - vl[v] > maxdeg) maxdeg = vl[v + 1] - vl[v];
    tw_pair* buf = (tw_pair*)malloc(sizeof(tw_pair) * (size_t)maxdeg);
    for (int32_t v = 0; v < V; ++v) {
        orow* o = &out[v];
        int32_t n = 0;
        for (int32_t e = vl[v]; e < vl[v + 1]; ++e)
            if (el[e] != v) buf[n].t = el[e], buf[n].w = wl[e], ++n;
        qsort(buf, (size_t)n, sizeof(tw_pair), ppr ? cmp_pair_float : cmp_pair_int);
        o->t = (int32_t*)malloc(sizeof(int32_t) * (size_t)(n ? n : 1));
        o->w = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(n ? n : 1));
        o->cap = n ? n : 1;
        o->n = 0;
        for (int32_t k = 0; k < n; ++k) {
            if (k > 0 && buf[k].t == buf[k - 1].t && buf[k].w == buf[k - 1].w) continue; /* equal pairs once */
            o->t[o->n] = buf[k].t;
            o->w[o->n] = buf[k].w;
            o->n++;
        }
        for (int32_t k = 0; k < o->n; ++k)
            if (k == 0 || o->t[k] != o->t[k - 1]) icnt[o->t[k]]++;
    }
    for (int32_t v = 0; v < V; ++v) {
        in[v].cap = icnt[v] ? icnt[v] : 1;
        in[v].n = 0;
        in[v].s = (int32_t*)malloc(sizeof(int32_t) * (size_t)in[v].cap);
        in[v].alive = (unsigned char*)malloc((size_t)in[v].cap);
    }
    for (int32_t v = 0; v < V; ++v) { /* sources in ascending order: rows stay sorted */
        const orow* o = &out[v];
        for (int32_t k = 0; k < o->n; ++k) {
            if (k > 0 && o->t[k] == o->t[k - 1]) continue;
            irow* r = &in[o->t[k]];
            r->s[r->n] = v;
            r->alive[r->n] = 1;
            r->n++;
        }
    }
    for (int32_t v = 0; v < V; ++v) indeg[v] = in[v].n;
    free(icnt);
    free(buf);
}

/* in-row position of source key (or the insertion point) */
static int32_t in_find(const irow* r, int32_t key) { return lower_i32(r->s, 0, r->n, key); }

static void in_insert(irow* r, int32_t at, int32_t src) {
    if (r->n == r->cap) {
        r->cap *= 2;
        r->s = (int32_t*)realloc(r->s, sizeof(int32_t) * (size_t)r->cap);
        r->alive = (unsigned char*)realloc(r->alive, (size_t)r->cap);
    }
    memmove(r->s + at + 1, r->s + at, sizeof(int32_t) * (size_t)(r->n - at));
    memmove(r->alive + at + 1, r->alive + at, (size_t)(r->n - at));
    r->s[at] = src;
    r->alive[at] = 1;
    r->n++;
}

typedef struct {
    ilist hv, he, hw, owner;
} records;

/* Dependency depth of a pruning order.  Every visit is an operation with read and write
 * sets over the rows it touches: the out-rows, and the in-rows with their live in-degree.
 * An operation's level is one more than the latest level that wrote a row it touches or
 * read a row it writes (read-after-write, write-after-read and write-after-write all
 * order two operations).  A visit includes its decision; the decision of a vertex that
 * is not pruned at its turn (its live in-degree out of bounds, or no out-edges) is an
 * operation of its own that reads the vertex's in-row and out-row.  The largest level is the length of the longest chain of
 * dependent operations: the fewest steps in which any parallel pruner that reproduces
 * the sequential bytes can run. */
typedef struct {
    int32_t *wo, *ro; /* out-row x: latest level that wrote / read it */
    int32_t *wi, *ri; /* in-row x (with the live in-degree) */
    int32_t depth;    /* largest level of any operation */
    int32_t pdepth;   /* largest level of a pruning visit */
    int64_t visits, removing, decisions;
    int64_t* width; /* pruning visits per level */
    int64_t width_cap;
} depth_track;

static int32_t imax(int32_t a, int32_t b) { return a > b ? a : b; }

static void depth_width(depth_track* d, int32_t lv) {
    if (lv >= d->width_cap) {
        int64_t cap = d->width_cap ? d->width_cap : 1024;
        while (cap <= lv) cap *= 2;
        d->width = (int64_t*)realloc(d->width, sizeof(int64_t) * (size_t)cap);
        memset(d->width + d->width_cap, 0, sizeof(int64_t) * (size_t)(cap - d->width_cap));
        d->width_cap = cap;
    }
    d->width[lv]++;
}

/* the visiting decision of vertex i: reads its in-row and out-row */
static void depth_decide(depth_track* d, int32_t i) {
    if (!d) return;
    const int32_t lv = 1 + imax(d->wi[i], d->wo[i]);
    d->ri[i] = imax(d->ri[i], lv);
    d->ro[i] = imax(d->ro[i], lv);
    d->depth = imax(d->depth, lv);
    d->decisions++;
}

/* Prune vertex i (src/purn-sssp.cpp:151-286, src/purn-ppr.cpp:154-284).  Returns 0, or
 * -3 when the in/out rows disagree (the reference prints "something error2"). */
static int prune_one(const prune_rule* rule, int32_t i, orow* out, irow* in, int32_t* indeg, records* rec,
                     depth_track* dt) {
    const int32_t j = indeg[i];
    int32_t* root = (int32_t*)malloc(sizeof(int32_t) * (size_t)(j ? j : 1));
    uint32_t* dis = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(j ? j : 1));
    int32_t* cur = (int32_t*)calloc((size_t)(j ? j : 1), sizeof(int32_t));
    int32_t* miss = (int32_t*)malloc(sizeof(int32_t) * (size_t)(j ? j : 1));
    int32_t nr = 0;
    /* roots: the live in-neighbours, with the weight of root -> i */
    for (int32_t k = 0; k < in[i].n; ++k) {
        if (!in[i].alive[k]) continue;
        const int32_t r = in[i].s[k];
        const orow* o = &out[r];
        const int32_t p = lower_i32(o->t, 0, o->n, i);
        if (p >= o->n || o->t[p] != i || nr >= j) {
            free(root), free(dis), free(cur), free(miss);
            return -3;
        }
        root[nr] = r;
        dis[nr] = o->w[p];
        ++nr;
    }
    if (nr != j) {
        free(root), free(dis), free(cur), free(miss);
        return -3;
    }
    orow* oi = &out[i];
    int32_t* kt = (int32_t*)malloc(sizeof(int32_t) * (size_t)(oi->n ? oi->n : 1));
    uint32_t* kw = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(oi->n ? oi->n : 1));
    int32_t* rt = (int32_t*)malloc(sizeof(int32_t) * (size_t)(oi->n ? oi->n : 1));
    uint32_t* rw = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(oi->n ? oi->n : 1));
    int32_t nk = 0, nrm = 0;
    for (int32_t e = 0; e < oi->n; ++e) {
        const int32_t v = oi->t[e];
        const uint32_t d3 = oi->w[e];
        int is_root = 0;
        for (int32_t k = 0; k < j; ++k)
            if (root[k] == v) is_root = 1;
        if (is_root) {
            kt[nk] = v, kw[nk] = d3, ++nk;
            continue;
        }
        int32_t cnt = 0, nm = 0;
        for (int32_t k = 0; k < j; ++k) {
            const orow* o = &out[root[k]];
            if (cur[k] + 1 < o->n && o->t[cur[k]] < v) cur[k] = lower_i32(o->t, cur[k], o->n - 1, v);
            if (o->t[cur[k]] == v)
                ++cnt;
            else
                miss[nm++] = root[k];
        }
        if (cnt + 2 > j) {
            rt[nrm] = v, rw[nrm] = d3, ++nrm;
            /* every root without r->v gains it: v's in-row gets r (alive) */
            for (int32_t m = 0; m < nm; ++m) {
                const int32_t r = miss[m];
                if (!rule->ppr && r == v) continue;
                irow* iv = &in[v];
                const int32_t p = in_find(iv, r);
                if (p >= iv->n || iv->s[p] != r) {
                    in_insert(iv, p, r);
                    indeg[v]++;
                } else if (!iv->alive[p]) {
                    iv->alive[p] = 1;
                    indeg[v]++;
                }
            }
            /* i -> v is gone: i dies in v's in-row */
            irow* iv = &in[v];
            const int32_t p = in_find(iv, i);
            if (p >= iv->n || iv->s[p] != i) {
                free(root), free(dis), free(cur), free(miss), free(kt), free(kw), free(rt), free(rw);
                return -3;
            }
            indeg[v]--;
            iv->alive[p] = 0;
        } else {
            kt[nk] = v, kw[nk] = d3, ++nk;
        }
    }
    if (dt) { /* reads: in-row i, out-rows of i and its roots; writes when edges move */
        int32_t lv = imax(dt->wi[i], dt->wo[i]);
        for (int32_t k = 0; k < j; ++k) lv = imax(lv, dt->wo[root[k]]);
        if (nrm > 0) {
            lv = imax(lv, imax(dt->ro[i], dt->ri[i]));
            for (int32_t k = 0; k < j; ++k) lv = imax(lv, dt->ro[root[k]]);
            for (int32_t k = 0; k < nrm; ++k) lv = imax(lv, imax(dt->wi[rt[k]], dt->ri[rt[k]]));
        }
        ++lv;
        dt->ri[i] = imax(dt->ri[i], lv);
        dt->ro[i] = imax(dt->ro[i], lv);
        for (int32_t k = 0; k < j; ++k) dt->ro[root[k]] = imax(dt->ro[root[k]], lv);
        if (nrm > 0) {
            dt->wo[i] = lv;
            for (int32_t k = 0; k < j; ++k) dt->wo[root[k]] = lv;
            for (int32_t k = 0; k < nrm; ++k) dt->wi[rt[k]] = lv;
            dt->removing++;
        }
        dt->depth = imax(dt->depth, lv);
        dt->pdepth = imax(dt->pdepth, lv);
        dt->visits++;
        depth_width(dt, lv);
    }
    /* fold the removed edges into every root's row (a sorted merge) */
    for (int32_t k = 0; k < j && nrm > 0; ++k) {
        orow* o = &out[root[k]];
        const int32_t cap = o->n + nrm;
        int32_t* nt = (int32_t*)malloc(sizeof(int32_t) * (size_t)cap);
        uint32_t* nw = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)cap);
        int32_t a = 0, b = 0, n = 0;
        while (a < o->n || b < nrm) {
            if (a < o->n && (b == nrm || o->t[a] < rt[b])) {
                nt[n] = o->t[a], nw[n] = o->w[a], ++n, ++a;
            } else if (a < o->n && o->t[a] == rt[b]) {
                nt[n] = o->t[a], nw[n] = fold_hit(rule, o->w[a], rw[b], dis[k]), ++n, ++a, ++b;
            } else { /* a new target from the record */
                if (!(!rule->ppr && rt[b] == root[k])) nt[n] = rt[b], nw[n] = fold_new(rule, rw[b], dis[k]), ++n;
                ++b;
            }
        }
        free(o->t);
        free(o->w);
        o->t = nt, o->w = nw, o->n = n, o->cap = cap;
    }
    free(oi->t);
    free(oi->w);
    oi->t = kt, oi->w = kw, oi->n = nk, oi->cap = oi->n ? oi->n : 1;
    for (int32_t k = 0; k < nrm; ++k) {
        il_push(&rec->he, (uint32_t)rt[k]);
        il_push(&rec->hw, rw[k]);
    }
    il_push(&rec->hv, (uint32_t)rec->he.n);
    il_push(&rec->owner, (uint32_t)i);
    free(root), free(dis), free(cur), free(miss), free(rt), free(rw);
    return 0;
}

static int prune_dir(const char* dir, int ppr, double keep, depth_track* dt) {
    size_t nv = 0, ne = 0, nw = 0;
    int32_t* vl = orc_read4(dir, "origin", "vlist", &nv);
    int32_t* el = orc_read4(dir, "origin", "elist", &ne);
    uint32_t* wl = (uint32_t*)orc_read4(dir, "origin", ppr ? "flist" : "wlist", &nw);
    if (!vl || !el || !wl || nv < 1 || nw < ne || (size_t)vl[nv - 1] != ne) {
        free(vl), free(el), free(wl);
        return -2;
    }
    const int32_t V = (int32_t)nv - 1;
    orow* out = (orow*)calloc((size_t)(V ? V : 1), sizeof(orow));
    irow* in = (irow*)calloc((size_t)(V ? V : 1), sizeof(irow));
    int32_t* indeg = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V ? V : 1));
    prune_rows(V, vl, el, wl, ppr, out, in, indeg);
    if (dt) {
        dt->wo = (int32_t*)calloc((size_t)(V ? V : 1), sizeof(int32_t));
        dt->ro = (int32_t*)calloc((size_t)(V ? V : 1), sizeof(int32_t));
        dt->wi = (int32_t*)calloc((size_t)(V ? V : 1), sizeof(int32_t));
        dt->ri = (int32_t*)calloc((size_t)(V ? V : 1), sizeof(int32_t));
    }
    free(el);
    free(wl);
    prune_rule rule = {ppr, keep};
    records rec;
    memset(&rec, 0, sizeof(rec));
    il_push(&rec.hv, 0);
    int rc = 0;
    if (!ppr) {
        const int32_t dmax = 29;
        unsigned char* seen = (unsigned char*)calloc((size_t)(V ? V : 1), 1);
        for (int32_t k = 0; k <= dmax && !rc; ++k)
            for (int32_t i = 0; i < V && !rc; ++i) {
                if (seen[i]) continue;
                if (indeg[i] > k || indeg[i] == 0) {
                    depth_decide(dt, i);
                    continue;
                }
                seen[i] = 1;
                if (out[i].n > 0 && indeg[i] > 0 && indeg[i] <= dmax)
                    rc = prune_one(&rule, i, out, in, indeg, &rec, dt);
                else
                    depth_decide(dt, i);
            }
        free(seen);
    } else {
        const int32_t dmax = 5;
        for (int32_t i = 0; i < V && !rc; ++i) {
            if (out[i].n > 0 && indeg[i] > 0 && indeg[i] <= dmax) {
                rc = prune_one(&rule, i, out, in, indeg, &rec, dt);
            } else {
                depth_decide(dt, i);
                il_push(&rec.hv, (uint32_t)rec.he.n);
                il_push(&rec.owner, (uint32_t)i);
            }
        }
    }
    if (!rc) {
        int64_t E = 0;
        for (int32_t v = 0; v < V; ++v) E += out[v].n;
        int32_t* pe = (int32_t*)malloc(sizeof(int32_t) * (size_t)(E ? E : 1));
        uint32_t* pw = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(E ? E : 1));
        int64_t e = 0;
        vl[0] = 0;
        for (int32_t v = 0; v < V; ++v) {
            memcpy(pe + e, out[v].t, sizeof(int32_t) * (size_t)out[v].n);
            memcpy(pw + e, out[v].w, sizeof(uint32_t) * (size_t)out[v].n);
            e += out[v].n;
            vl[v + 1] = (int32_t)e;
        }
        const char* sub = ppr ? "ppr" : "sssp";
        char p[4096];
        snprintf(p, sizeof(p), "%s/%s", dir, sub);
        rc = orc_mkdir(p);
        if (!rc) rc = orc_write4(dir, sub, "hvlist", rec.hv.a, (size_t)rec.hv.n);
        if (!rc) rc = orc_write4(dir, sub, "helist", rec.he.a, (size_t)rec.he.n);
        if (!rc) rc = orc_write4(dir, sub, "hwlist", rec.hw.a, (size_t)rec.hw.n);
        if (!rc && !ppr) rc = orc_write4(dir, sub, "hvmap", rec.owner.a, (size_t)rec.owner.n);
        if (!rc) rc = orc_write4(dir, sub, "vlist", vl, (size_t)V + 1);
        if (!rc) rc = orc_write4(dir, sub, "elist", pe, (size_t)E);
        if (!rc) rc = orc_write4(dir, sub, "wlist", pw, (size_t)E);
        free(pe);
        free(pw);
    }
    for (int32_t v = 0; v < V; ++v) {
        free(out[v].t), free(out[v].w);
        free(in[v].s), free(in[v].alive);
    }
    free(out), free(in), free(indeg), free(vl);
    if (dt) free(dt->wo), free(dt->ro), free(dt->wi), free(dt->ri);
    free(rec.hv.a), free(rec.he.a), free(rec.hw.a), free(rec.owner.a);
    return rc;
}

int orc_prune_sssp(const char* dir) { return dir ? prune_dir(dir, 0, 0.0, NULL) : -1; }

/* keep = 1 - alpha of the push the pruned graph serves; 0.8 is the reference's */
int orc_prune_ppr(const char* dir, double keep) { return dir ? prune_dir(dir, 1, keep, NULL) : -1; }

/* The pruner of kind ppr (0: purn-sssp, 1: purn-ppr with keep) with the dependency
 * analysis above; its outputs are written as by orc_prune_sssp / orc_prune_ppr.  st[8]:
 * pruning visits, visits that moved edges, visiting decisions, depth over all operations,
 * depth over the pruning visits, the widest level's visits, and the visits that sit in
 * levels of at least 32 and of at least 1024 visits. */
int orc_prune_depth(const char* dir, int ppr, double keep, int64_t* st) {
    if (!dir || !st) return -1;
    depth_track d;
    memset(&d, 0, sizeof(d));
    const int rc = prune_dir(dir, ppr ? 1 : 0, keep, &d);
    int64_t wmax = 0, w32 = 0, w1k = 0;
    for (int64_t l = 0; l < d.width_cap; ++l) {
        const int64_t w = d.width[l];
        if (w > wmax) wmax = w;
        if (w >= 32) w32 += w;
        if (w >= 1024) w1k += w;
    }
    st[0] = d.visits, st[1] = d.removing, st[2] = d.decisions, st[3] = d.depth, st[4] = d.pdepth;
    st[5] = wmax, st[6] = w32, st[7] = w1k;
    free(d.width);
    return rc;
}

/* ---- a parallel schedule of the pruners, checked on the CPU ----------------------------
 * The pruners visit positions (k, i) in order: purn-ppr one per vertex (bound 5), purn-sssp
 * one per round k = 1..29 and vertex (a vertex is visited at the first k that covers its live
 * in-degree).  orc_prune_speculative runs the same steps (prune_one, unchanged) in rounds over
 * a window of `window` positions from the first pending one, the schedule of the device
 * pruners (deterministic reservations): each pending position computes, on the current
 * state, the rows it reads (its in-row, its out-row, its live roots' out-rows) and the rows it
 * would write (its out-row and its roots' out-rows when it moves edges, the in-rows of the
 * targets it moves); it reserves them under its index; it commits when no earlier position
 * of the window writes a row it reads and none touches a row it writes.  A position with an
 * earlier writer of a row it reads has a plan that may change before it commits (whether
 * that writer commits in this round or a later one), and so may the rows it will touch:
 * positions past the first such one wait.  Records are
 * gathered per vertex and written in visiting order (purn-ppr: id order; purn-sssp: (k, id),
 * with the record->vertex sidecar).  The outputs go to dir/<sub>/ in the ppr/ or sssp/
 * layout, so a test compares them byte by byte with orc_prune_ppr's / orc_prune_sssp's.
 * st[3]: rounds, committed positions, the largest round. */
typedef struct {
    int32_t* a;
    int32_t n, cap;
} rowset;

static void rs_push(rowset* v, int32_t x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 16;
        v->a = (int32_t*)realloc(v->a, sizeof(int32_t) * (size_t)v->cap);
    }
    v->a[v->n++] = x;
}

/* rows of position (k, i) on the current state: out-row x is x, in-row x is V + x */
static void visit_rows(int32_t i, int32_t k, int32_t V, const orow* out, const irow* in, const int32_t* indeg,
                       rowset* R, rowset* W) {
    R->n = W->n = 0;
    rs_push(R, V + i);
    rs_push(R, i);
    if (!(out[i].n > 0 && indeg[i] > 0 && indeg[i] <= k)) return;
    int32_t root[32], nr = 0, cur[32] = {0};
    for (int32_t q = 0; q < in[i].n; ++q)
        if (in[i].alive[q] && nr < 32) root[nr++] = in[i].s[q];
    const int32_t j = indeg[i] < nr ? indeg[i] : nr;
    for (int32_t q = 0; q < nr; ++q) rs_push(R, root[q]);
    int moves = 0;
    const orow* oi = &out[i];
    for (int32_t e = 0; e < oi->n; ++e) { /* the decisions of prune_one, without its writes */
        const int32_t v = oi->t[e];
        int is_root = 0;
        for (int32_t q = 0; q < j; ++q)
            if (root[q] == v) is_root = 1;
        if (is_root) continue;
        int32_t cnt = 0;
        for (int32_t q = 0; q < j; ++q) {
            const orow* o = &out[root[q]];
            if (cur[q] + 1 < o->n && o->t[cur[q]] < v) cur[q] = lower_i32(o->t, cur[q], o->n - 1, v);
            if (o->t[cur[q]] == v) ++cnt;
        }
        if (cnt + 2 > j) {
            rs_push(W, V + v);
            moves = 1;
        }
    }
    if (moves) {
        rs_push(W, i);
        for (int32_t q = 0; q < nr; ++q) rs_push(W, root[q]);
    }
}

int orc_prune_speculative(const char* dir, int ppr, double keep, int32_t window, const char* sub, int64_t* st) {
    if (!dir || !sub || !st || window < 1) return -1;
    size_t nv = 0, ne = 0, nw = 0;
    int32_t* vl = orc_read4(dir, "origin", "vlist", &nv);
    int32_t* el = orc_read4(dir, "origin", "elist", &ne);
    uint32_t* wl = (uint32_t*)orc_read4(dir, "origin", ppr ? "flist" : "wlist", &nw);
    if (!vl || !el || !wl || nv < 1 || nw < ne || (size_t)vl[nv - 1] != ne) {
        free(vl), free(el), free(wl);
        return -2;
    }
    const int32_t V = (int32_t)nv - 1;
    const int32_t kfirst = ppr ? 5 : 1, klast = ppr ? 5 : 29;
    const int64_t npos = (int64_t)(klast - kfirst + 1) * V;
    if (window > V) window = V ? V : 1; /* no vertex twice in a window */
    orow* out = (orow*)calloc((size_t)(V ? V : 1), sizeof(orow));
    irow* in = (irow*)calloc((size_t)(V ? V : 1), sizeof(irow));
    int32_t* indeg = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V ? V : 1));
    prune_rows(V, vl, el, wl, ppr, out, in, indeg);
    free(el);
    free(wl);
    const prune_rule rule = {ppr, keep};
    int32_t* pk = (int32_t*)malloc(sizeof(int32_t) * (size_t)(V ? V : 1)); /* last round done per vertex */
    int32_t* vk = (int32_t*)calloc((size_t)(V ? V : 1), sizeof(int32_t));  /* round of the pruning visit */
    for (int32_t v = 0; v < V; ++v) pk[v] = kfirst - 1;
    int64_t* resA = (int64_t*)calloc(2 * (size_t)(V ? V : 1), sizeof(int64_t)); /* (round << 32) | ~pos: max wins */
    int64_t* resW = (int64_t*)calloc(2 * (size_t)(V ? V : 1), sizeof(int64_t));
    rowset* R = (rowset*)calloc((size_t)window, sizeof(rowset));
    rowset* W = (rowset*)calloc((size_t)window, sizeof(rowset));
    int64_t* cand = (int64_t*)malloc(sizeof(int64_t) * (size_t)window);
    unsigned char* pass = (unsigned char*)malloc((size_t)window);
    int64_t* rec_off = (int64_t*)calloc((size_t)V + 1, sizeof(int64_t)); /* per-vertex records, in commit order */
    int32_t* rec_n = (int32_t*)calloc((size_t)(V ? V : 1), sizeof(int32_t));
    ilist pool_t, pool_w;
    memset(&pool_t, 0, sizeof(pool_t));
    memset(&pool_w, 0, sizeof(pool_w));
    records one;
    memset(&one, 0, sizeof(one));
    int64_t pos = 0, commits = 0;
    int32_t rounds = 0, widest = 0;
    int rc = 0;
#define POS_K(p) (kfirst + (int32_t)((p) / V))
#define POS_I(p) ((int32_t)((p) % V))
    while (pos < npos && !rc) {
        ++rounds;
        int32_t n = 0;
        for (int64_t p = pos; p < npos && p < pos + window; ++p)
            if (pk[POS_I(p)] < POS_K(p)) cand[n++] = p;
        const int64_t tag = (int64_t)rounds << 32;
        for (int32_t c = 0; c < n; ++c) { /* plan and reserve */
            visit_rows(POS_I(cand[c]), POS_K(cand[c]), V, out, in, indeg, &R[c], &W[c]);
            const int64_t key = tag | (int64_t)(uint32_t)~(uint32_t)cand[c];
            for (int32_t q = 0; q < R[c].n; ++q)
                if (resA[R[c].a[q]] < key) resA[R[c].a[q]] = key;
            for (int32_t q = 0; q < W[c].n; ++q) {
                if (resA[W[c].a[q]] < key) resA[W[c].a[q]] = key;
                if (resW[W[c].a[q]] < key) resW[W[c].a[q]] = key;
            }
        }
        int64_t dmin = npos; /* the first position with an earlier writer of a row it reads */
        for (int32_t c = 0; c < n; ++c) { /* check */
            const int64_t key = tag | (int64_t)(uint32_t)~(uint32_t)cand[c];
            int wok = 1, rok = 1;
            for (int32_t q = 0; q < W[c].n && wok; ++q)
                if (resA[W[c].a[q]] != key) wok = 0; /* an earlier position touches a row it writes */
            for (int32_t q = 0; q < R[c].n && rok; ++q)
                if (resW[R[c].a[q]] > key) rok = 0; /* an earlier position writes a row it reads */
            pass[c] = (unsigned char)(wok && rok);
            if (!rok && cand[c] < dmin) dmin = cand[c];
        }
        int32_t nc = 0;
        for (int32_t c = 0; c < n && !rc; ++c) { /* commit */
            if (!pass[c] || cand[c] > dmin) continue;
            const int32_t i = POS_I(cand[c]), k = POS_K(cand[c]);
            /* a vertex whose live in-degree is 0 or above k is skipped; the rest are
             * visited, and pruned when the in-degree is positive and out-edges remain */
            const int visit = indeg[i] != 0 && indeg[i] <= k;
            if (visit && indeg[i] > 0 && out[i].n > 0) {
                one.he.n = one.hw.n = one.hv.n = one.owner.n = 0;
                il_push(&one.hv, 0);
                if (prune_one(&rule, i, out, in, indeg, &one, NULL)) rc = -3;
                rec_off[i] = pool_t.n;
                rec_n[i] = (int32_t)one.he.n;
                vk[i] = k;
                for (int64_t q = 0; q < one.he.n; ++q) {
                    il_push(&pool_t, one.he.a[q]);
                    il_push(&pool_w, one.hw.a[q]);
                }
            }
            pk[i] = visit ? klast : k;
            ++nc;
        }
        commits += nc;
        if (nc > widest) widest = nc;
        while (pos < npos && pk[POS_I(pos)] >= POS_K(pos)) ++pos;
    }
#undef POS_K
#undef POS_I
    if (!rc) {
        /* records in visiting order: purn-ppr one per vertex, purn-sssp one per pruned vertex
         * in (round, id) order with the sidecar */
        records rec;
        memset(&rec, 0, sizeof(rec));
        il_push(&rec.hv, 0);
        for (int32_t k = ppr ? 0 : 1; k <= (ppr ? 0 : klast); ++k)
            for (int32_t v = 0; v < V; ++v) {
                if (!ppr && vk[v] != k) continue;
                for (int32_t q = 0; q < rec_n[v]; ++q) {
                    il_push(&rec.he, pool_t.a[rec_off[v] + q]);
                    il_push(&rec.hw, pool_w.a[rec_off[v] + q]);
                }
                il_push(&rec.hv, (uint32_t)rec.he.n);
                il_push(&rec.owner, (uint32_t)v);
            }
        int64_t E = 0;
        for (int32_t v = 0; v < V; ++v) E += out[v].n;
        int32_t* pe = (int32_t*)malloc(sizeof(int32_t) * (size_t)(E ? E : 1));
        uint32_t* pw = (uint32_t*)malloc(sizeof(uint32_t) * (size_t)(E ? E : 1));
        int64_t e = 0;
        vl[0] = 0;
        for (int32_t v = 0; v < V; ++v) {
            memcpy(pe + e, out[v].t, sizeof(int32_t) * (size_t)out[v].n);
            memcpy(pw + e, out[v].w, sizeof(uint32_t) * (size_t)out[v].n);
            e += out[v].n;
            vl[v + 1] = (int32_t)e;
        }
        char p[4096];
        snprintf(p, sizeof(p), "%s/%s", dir, sub);
        rc = orc_mkdir(p);
        if (!rc) rc = orc_write4(dir, sub, "hvlist", rec.hv.a, (size_t)rec.hv.n);
        if (!rc) rc = orc_write4(dir, sub, "helist", rec.he.a, (size_t)rec.he.n);
        if (!rc) rc = orc_write4(dir, sub, "hwlist", rec.hw.a, (size_t)rec.hw.n);
        if (!rc && !ppr) rc = orc_write4(dir, sub, "hvmap", rec.owner.a, (size_t)rec.owner.n);
        if (!rc) rc = orc_write4(dir, sub, "vlist", vl, (size_t)V + 1);
        if (!rc) rc = orc_write4(dir, sub, "elist", pe, (size_t)E);
        if (!rc) rc = orc_write4(dir, sub, "wlist", pw, (size_t)E);
        free(pe), free(pw), free(rec.hv.a), free(rec.he.a), free(rec.hw.a), free(rec.owner.a);
    }
    st[0] = rounds, st[1] = commits, st[2] = widest;
    for (int32_t v = 0; v < V; ++v) {
        free(out[v].t), free(out[v].w);
        free(in[v].s), free(in[v].alive);
    }
    for (int32_t c = 0; c < window; ++c) free(R[c].a), free(W[c].a);
    free(out), free(in), free(indeg), free(vl), free(pk), free(vk), free(resA), free(resW), free(R), free(W);
    free(cand), free(pass), free(rec_off), free(rec_n), free(pool_t.a), free(pool_w.a);
    free(one.hv.a), free(one.he.a), free(one.hw.a), free(one.owner.a);
    return rc;
}

/* purn-ppr's schedule check (the first user of orc_prune_speculative) */
int orc_prune_ppr_speculative(const char* dir, double keep, int32_t window, const char* sub, int64_t* st) {
    return orc_prune_speculative(dir, 1, keep, window, sub, st);
}
