// C^2graph-P offline pruners, written to produce the same bytes as the reference's
// purn-sssp (src/purn-sssp.cpp:61-352) and purn-ppr (src/purn-ppr.cpp:63-344).
//
// Both prune edges out of low-in-degree vertices i: an out-edge i->v is removed when
// every live in-neighbour ("root") r of i, except at most one, already has an edge to
// v.  The missing root gets r->v, every root's r->v weight is combined with the path
// through i, and the removed edges of i are appended as one "record" (hvlist/helist/
// hwlist) that the traversal uses as seeds when i is the source.
//
// The pruning is sequential by construction: the order in which vertices are visited
// changes which edges survive, so this stays a single-threaded host pass.  What this
// file adds over the reference is the record->vertex sidecar sssp/hvmap.bin: purn-sssp
// appends records in pruning order (rounds k = 0..29 over all vertices), while the
// traversal indexes hvlist by vertex id (src/sssp/purn/Main.cu:68-79).
#include <algorithm>
#include <cstring>
#include <cstdint>
#include <memory>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

#include <omp.h>

#include "../../include/c2graph.h"
#include "host_io.h"

namespace c2g {

namespace {

template <typename W>
using Adj = std::vector<std::vector<std::pair<int32_t, W>>>;
using InAdj = std::vector<std::vector<std::pair<int32_t, bool>>>;

std::vector<std::pair<int32_t, bool>>::iterator in_find(std::vector<std::pair<int32_t, bool>>& row,
                                                         int32_t key) {
    return std::lower_bound(row.begin(), row.end(), key,
                            [](const std::pair<int32_t, bool>& a, int32_t b) { return a.first < b; });
}

// Weight rules of the two pruners.
struct SsspRule {
    using W = int32_t;
    static W combine_new(W d3, W dis) { return d3 + dis; }
    static W combine_hit(W old, W d3, W dis) { return std::min(old, d3 + dis); }
    static constexpr bool skip_root_target = true;  // src/purn-sssp.cpp:244,263
};
// Factor of a folded PPR edge: the continuation probability 1 - alpha of the push the
// pruned graph is built for.  The reference bakes 0.8 (alpha 0.2) into it.
thread_local double g_ppr_keep = 0.8;

struct PprRule {
    using W = float;
    // (float * keep) * float evaluated in double, then rounded to float, keep = 0.8 in
    // the reference (src/purn-ppr.cpp:244,255,259).
    static W combine_new(W d3, W dis) { return (float)((double)d3 * g_ppr_keep * (double)dis); }
    static W combine_hit(W old, W d3, W dis) {
        return (float)((double)old + (double)d3 * g_ppr_keep * (double)dis);
    }
    static constexpr bool skip_root_target = false;
};

struct Records {
    std::vector<int32_t> hv{0};
    std::vector<int32_t> he;
    std::vector<int32_t> hw_i;
    std::vector<float> hw_f;
    std::vector<int32_t> owner;  // record -> vertex
};

// Prune vertex i (its in-degree is within the pruner's bound).  Appends i's record.
template <typename R>
int prune_vertex(int32_t i, Adj<typename R::W>& out, InAdj& in, std::vector<int32_t>& indeg,
                 Records& rec) {
    using W = typename R::W;
    std::vector<int32_t> roots;
    std::vector<W> dis;
    for (auto& p : in[i]) {
        if (!p.second) continue;
        const int32_t r = p.first;
        auto& orow = out[r];
        auto it = std::lower_bound(orow.begin(), orow.end(), i,
                                   [](const std::pair<int32_t, W>& a, int32_t b) { return a.first < b; });
        if (it == orow.end() || it->first != i)
            return fail(C2G_ERR_FORMAT, "prune: live in-edge %d->%d has no out-edge", r, i);
        roots.push_back(r);
        dis.push_back(it->second);
    }
    const size_t j = roots.size();
    if ((int64_t)j != indeg[i])
        return fail(C2G_ERR_FORMAT, "prune: vertex %d live in-degree %d != %zu roots", i, indeg[i], j);

    std::vector<size_t> cursor(j, 0);
    std::vector<std::pair<int32_t, W>> kept, removed;
    std::vector<int32_t> missing;
    for (const auto& ev : out[i]) {
        const int32_t v = ev.first;
        if (std::find(roots.begin(), roots.end(), v) != roots.end()) {
            kept.push_back(ev);
            continue;
        }
        size_t cnt = 0;
        missing.clear();
        for (size_t k = 0; k < j; ++k) {
            const auto& orow = out[roots[k]];
            // Monotone cursor over the root's sorted row: the first position at or after
            // the cursor whose target is >= v, or the row's last element
            // (src/purn-sssp.cpp:198-200).  Binary search gives the same position as the
            // reference's linear walk.
            if (cursor[k] + 1 < orow.size() && orow[cursor[k]].first < v) {
                auto it = std::lower_bound(orow.begin() + (long)cursor[k], orow.end() - 1, v,
                                           [](const std::pair<int32_t, W>& a, int32_t b) { return a.first < b; });
                cursor[k] = (size_t)(it - orow.begin());
            }
            if (orow[cursor[k]].first == v)
                ++cnt;
            else
                missing.push_back(roots[k]);
        }
        if (cnt + 2 > j) {
            removed.push_back(ev);
            for (int32_t r : missing) {
                if (R::skip_root_target && r == v) continue;
                auto& irow = in[v];
                auto it = in_find(irow, r);
                if (it == irow.end() || it->first != r) {
                    irow.insert(it, std::make_pair(r, true));
                    indeg[v]++;
                } else if (!it->second) {
                    indeg[v]++;
                    it->second = true;
                }
            }
            auto it = in_find(in[v], i);
            if (it == in[v].end() || it->first != i)
                return fail(C2G_ERR_FORMAT, "prune: edge %d->%d missing from in-list", i, v);
            indeg[v]--;
            it->second = false;
        } else {
            kept.push_back(ev);
        }
    }

    // Merge the removed edges into every root's row with the combined weight (a merge
    // of nothing leaves a row unchanged, so it is skipped).
    std::vector<std::pair<int32_t, W>> merged;
    for (size_t k = 0; k < j && !removed.empty(); ++k) {
        const int32_t r = roots[k];
        auto& orow = out[r];
        merged.clear();
        merged.reserve(orow.size() + removed.size());
        size_t a = 0, b = 0;
        while (a < orow.size() || b < removed.size()) {
            if (a == orow.size()) {
                if (R::skip_root_target && removed[b].first == r) { ++b; continue; }
                merged.emplace_back(removed[b].first, R::combine_new(removed[b].second, dis[k]));
                ++b;
            } else if (b == removed.size()) {
                merged.push_back(orow[a++]);
            } else if (orow[a].first == removed[b].first) {
                merged.emplace_back(orow[a].first, R::combine_hit(orow[a].second, removed[b].second, dis[k]));
                ++a;
                ++b;
            } else if (orow[a].first > removed[b].first) {
                if (R::skip_root_target && removed[b].first == r) { ++b; continue; }
                merged.emplace_back(removed[b].first, R::combine_new(removed[b].second, dis[k]));
                ++b;
            } else {
                merged.push_back(orow[a++]);
            }
        }
        orow.swap(merged);
    }
    out[i].swap(kept);

    for (const auto& ev : removed) {
        rec.he.push_back(ev.first);
        if constexpr (std::is_same<W, float>::value)
            rec.hw_f.push_back(ev.second);
        else
            rec.hw_i.push_back(ev.second);
    }
    rec.hv.push_back(rec.hv.back() + (int32_t)removed.size());
    rec.owner.push_back(i);
    return C2G_OK;
}

template <typename W>
void flatten(const Adj<W>& out, int32_t V, std::vector<int32_t>& vlist, std::vector<int32_t>& elist,
             std::vector<W>& wl) {
    vlist.assign((size_t)V + 1, 0);
    size_t E = 0;
    for (int32_t v = 0; v < V; ++v) E += out[v].size();
    elist.resize(E);
    wl.resize(E);
    size_t e = 0;
    for (int32_t v = 0; v < V; ++v) {
        for (const auto& p : out[v]) {
            elist[e] = p.first;
            wl[e] = p.second;
            ++e;
        }
        vlist[v + 1] = (int32_t)e;
    }
}

}  // namespace

// The rows a pruner starts from, flat, for the device pruners (prune_gpu.cu) and the host
// passes: out-rows of the (target, weight) pairs without self-loops, sorted as
// pair<int32, W> and without repeated pairs (the reference builds them through std::set,
// core/util.hpp:94-110); in-rows of the distinct sources of each vertex, ascending.  Built
// without one allocation per row.  Input rows that are
// already strictly increasing and free of self-loops (the R-MAT writer's) are the out-rows
// as they are; other rows are sorted in parallel.  The in-rows are a stable counting sort
// of the out-rows by target, each thread filling its own range of sources.  orow / irow are
// row pointers over V + 1 entries.  W is float (purn-ppr: origin/flist.bin) or int32
// (purn-sssp: origin/wlist.bin).
template <typename W>
int prune_initial_rows(const std::string& dir, int32_t& V, std::vector<int32_t>& orow, std::vector<int32_t>& ot,
                       std::vector<W>& ow, std::vector<int32_t>& irow, std::vector<int32_t>& is) {
    constexpr bool kFloat = std::is_same<W, float>::value;
    std::vector<int32_t> vlist, elist;
    std::vector<W> flist;
    int rc;
    if ((rc = read_array4(dir + "/origin/vlist.bin", vlist))) return rc;
    if ((rc = read_array4(dir + "/origin/elist.bin", elist))) return rc;
    if ((rc = read_array4(dir + (kFloat ? "/origin/flist.bin" : "/origin/wlist.bin"), flist))) return rc;
    if ((rc = check_csr(vlist, elist))) return rc;
    if (flist.size() < elist.size()) return fail(C2G_ERR_FORMAT, kFloat ? "flist shorter than elist" : "wlist shorter than elist");
    V = (int32_t)vlist.size() - 1;
    int plain = 1;
#pragma omp parallel for schedule(dynamic, 4096) reduction(& : plain)
    for (int32_t v = 0; v < V; ++v)
        for (int32_t e = vlist[v]; e < vlist[v + 1]; ++e)
            if (elist[e] == v || (e > vlist[v] && elist[e] <= elist[e - 1])) plain = 0;
    if (plain) {
        orow = vlist;
        flist.resize(elist.size());
        ot = std::move(elist);
        ow = std::move(flist);
    } else {
        std::vector<std::pair<int32_t, W>> pr(elist.size());
        std::vector<int32_t> cnt((size_t)V, 0);
#pragma omp parallel for schedule(dynamic, 4096)
        for (int32_t v = 0; v < V; ++v) {
            auto* row = pr.data() + vlist[v];
            int32_t k = 0;
            for (int32_t e = vlist[v]; e < vlist[v + 1]; ++e)
                if (elist[e] != v) row[k++] = std::make_pair(elist[e], flist[e]);
            std::sort(row, row + k);
            cnt[v] = (int32_t)(std::unique(row, row + k) - row);
        }
        orow.assign((size_t)V + 1, 0);
        for (int32_t v = 0; v < V; ++v) orow[v + 1] = orow[v] + cnt[v];
        ot.resize((size_t)orow[V]);
        ow.resize((size_t)orow[V]);
#pragma omp parallel for schedule(dynamic, 4096)
        for (int32_t v = 0; v < V; ++v) {
            const auto* row = pr.data() + vlist[v];
            for (int32_t x = 0; x < cnt[v]; ++x) {
                ot[(size_t)orow[v] + x] = row[x].first;
                ow[(size_t)orow[v] + x] = row[x].second;
            }
        }
    }
    // in-rows: thread t counts, then fills, the distinct targets of sources [V t / T, V (t+1) / T)
    const int T = std::max(1, std::min(omp_get_max_threads(), 64));
    std::unique_ptr<int32_t[]> c(new int32_t[(size_t)T * (size_t)V + 1]);
    irow.assign((size_t)V + 1, 0);
    auto distinct = [&](int32_t v, size_t x) { return x == (size_t)orow[v] || ot[x] != ot[x - 1]; };
#pragma omp parallel num_threads(T)
    {
        const int t = omp_get_thread_num();
        int32_t* ct = c.get() + (size_t)t * V;
        std::fill(ct, ct + V, 0);
        const int32_t v0 = (int32_t)((int64_t)V * t / T), v1 = (int32_t)((int64_t)V * (t + 1) / T);
        for (int32_t v = v0; v < v1; ++v)
            for (size_t x = (size_t)orow[v]; x < (size_t)orow[v + 1]; ++x)
                if (distinct(v, x)) ++ct[ot[x]];
#pragma omp barrier
#pragma omp for schedule(static)
        for (int32_t d = 0; d < V; ++d) {
            int32_t n = 0;
            for (int u = 0; u < T; ++u) n += c[(size_t)u * V + d];
            irow[(size_t)d + 1] = n;
        }
#pragma omp single
        for (int32_t d = 0; d < V; ++d) irow[(size_t)d + 1] += irow[d];
#pragma omp for schedule(static)
        for (int32_t d = 0; d < V; ++d) {
            int32_t run = irow[d];
            for (int u = 0; u < T; ++u) {
                const int32_t k = c[(size_t)u * V + d];
                c[(size_t)u * V + d] = run;
                run += k;
            }
        }
#pragma omp single
        is.resize((size_t)irow[V]);
        for (int32_t v = v0; v < v1; ++v)
            for (size_t x = (size_t)orow[v]; x < (size_t)orow[v + 1]; ++x)
                if (distinct(v, x)) is[(size_t)ct[ot[x]]++] = v;
    }
    return C2G_OK;
}

template int prune_initial_rows<float>(const std::string&, int32_t&, std::vector<int32_t>&, std::vector<int32_t>&,
                                      std::vector<float>&, std::vector<int32_t>&, std::vector<int32_t>&);
template int prune_initial_rows<int32_t>(const std::string&, int32_t&, std::vector<int32_t>&, std::vector<int32_t>&,
                                        std::vector<int32_t>&, std::vector<int32_t>&, std::vector<int32_t>&);

namespace {

// The host passes' per-vertex rows (every in-entry alive), filled from the flat initial rows.
template <typename W>
int host_rows(const std::string& dir, int32_t& V, Adj<W>& out, InAdj& in, std::vector<int32_t>& indeg) {
    std::vector<int32_t> orow, ot, irow, is;
    std::vector<W> ow;
    const int rc = prune_initial_rows<W>(dir, V, orow, ot, ow, irow, is);
    if (rc) return rc;
    out.assign((size_t)V, {});
    in.assign((size_t)V, {});
    indeg.assign((size_t)V, 0);
#pragma omp parallel for schedule(dynamic, 4096)
    for (int32_t v = 0; v < V; ++v) {
        auto& o = out[v];
        o.reserve((size_t)(orow[v + 1] - orow[v]));
        for (int32_t x = orow[v]; x < orow[v + 1]; ++x) o.emplace_back(ot[x], ow[x]);
        auto& r = in[v];
        r.reserve((size_t)(irow[v + 1] - irow[v]));
        for (int32_t x = irow[v]; x < irow[v + 1]; ++x) r.emplace_back(is[x], true);
        indeg[v] = irow[v + 1] - irow[v];
    }
    return C2G_OK;
}

}  // namespace

int prune_sssp_dir(const std::string& dir) {
    int32_t V = 0;
    Adj<int32_t> out;
    InAdj in;
    std::vector<int32_t> indeg;
    int rc = host_rows<int32_t>(dir, V, out, in, indeg);
    if (rc) return rc;

    // Rounds k = 0..29; a vertex is visited once, in the first round whose bound
    // covers its live in-degree (src/purn-sssp.cpp:139-150).
    const int32_t dmax = 29;
    Records rec;
    std::vector<char> visited(V, 0);
    for (int32_t k = 0; k <= dmax; ++k) {
        for (int32_t i = 0; i < V; ++i) {
            if (indeg[i] > k || visited[i] || indeg[i] == 0) continue;
            visited[i] = 1;
            if (!out[i].empty() && indeg[i] > 0 && indeg[i] <= dmax)
                if ((rc = prune_vertex<SsspRule>(i, out, in, indeg, rec))) return rc;
        }
    }
    InAdj().swap(in);
    std::vector<int32_t> pv, pe, pw;
    flatten(out, V, pv, pe, pw);
    const std::string s = dir + "/sssp/";
    if ((rc = make_dir(dir + "/sssp"))) return rc;
    if ((rc = write_array4(s + "hvlist.bin", rec.hv.data(), rec.hv.size()))) return rc;
    if ((rc = write_array4(s + "helist.bin", rec.he.data(), rec.he.size()))) return rc;
    if ((rc = write_array4(s + "hwlist.bin", rec.hw_i.data(), rec.hw_i.size()))) return rc;
    if ((rc = write_array4(s + "hvmap.bin", rec.owner.data(), rec.owner.size()))) return rc;
    if ((rc = write_array4(s + "vlist.bin", pv.data(), pv.size()))) return rc;
    if ((rc = write_array4(s + "elist.bin", pe.data(), pe.size()))) return rc;
    if ((rc = write_array4(s + "wlist.bin", pw.data(), pw.size()))) return rc;
    return C2G_OK;
}

int prune_ppr_dir(const std::string& dir, double keep) {
    g_ppr_keep = keep;
    int32_t V = 0;
    Adj<float> out;
    InAdj in;
    std::vector<int32_t> indeg;
    int rc = host_rows<float>(dir, V, out, in, indeg);
    if (rc) return rc;

    // One pass in vertex order with in-degree bound 5; every vertex gets a record,
    // empty when it is not pruned (src/purn-ppr.cpp:146-152,281-283).
    const int32_t dmax = 5;
    Records rec;
    for (int32_t i = 0; i < V; ++i) {
        if (!out[i].empty() && indeg[i] > 0 && indeg[i] <= dmax) {
            if ((rc = prune_vertex<PprRule>(i, out, in, indeg, rec))) return rc;
        } else {
            rec.hv.push_back(rec.hv.back());
            rec.owner.push_back(i);
        }
    }
    InAdj().swap(in);
    std::vector<int32_t> pv, pe;
    std::vector<float> pw;
    flatten(out, V, pv, pe, pw);
    const std::string s = dir + "/ppr/";
    if ((rc = make_dir(dir + "/ppr"))) return rc;
    if ((rc = write_array4(s + "hvlist.bin", rec.hv.data(), rec.hv.size()))) return rc;
    if ((rc = write_array4(s + "helist.bin", rec.he.data(), rec.he.size()))) return rc;
    if ((rc = write_array4(s + "hwlist.bin", rec.hw_f.data(), rec.hw_f.size()))) return rc;
    if ((rc = write_array4(s + "vlist.bin", pv.data(), pv.size()))) return rc;
    if ((rc = write_array4(s + "elist.bin", pe.data(), pe.size()))) return rc;
    if ((rc = write_array4(s + "wlist.bin", pw.data(), pw.size()))) return rc;
    return C2G_OK;
}

}  // namespace c2g

extern "C" int c2g_prune_sssp(const char* dir) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "prune: dir is NULL");
    return c2g::prune_sssp_dir(dir);
}

extern "C" int c2g_prune_ppr(const char* dir) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "prune: dir is NULL");
    return c2g::prune_ppr_dir(dir, 0.8);
}

extern "C" int c2g_prune_ppr_alpha(const char* dir, double alpha) {
    if (!dir) return c2g::fail(C2G_ERR_ARG, "prune: dir is NULL");
    if (!(alpha > 0.0 && alpha < 1.0)) return c2g::fail(C2G_ERR_ARG, "prune: alpha must be in (0, 1)");
    return c2g::prune_ppr_dir(dir, 1.0 - alpha);
}
