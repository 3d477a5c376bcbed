"""Generate the golden fixtures in tests/golden/ from the reference's own code.

Run where the reference tree is mounted (it builds oracle/_ref/ from the reference
sources first):   python tests/golden/make_golden.py

For every case it writes <case>.npz holding
  origin_*      the input graph (reference origin/ layout)
  sssp_*, ppr_* the outputs of the reference purn-sssp / purn-ppr on that input
  hvmap         record -> vertex order of the sssp records (from this library's
                pruner, whose other outputs must equal the reference's byte for byte)
  dist_origin   reference CPU Bellman-Ford (ref-bf) distances on origin/ per source
  dist_compat   ref-bf on sssp/ seeded from hvlist indexed by the source (sssp-purn)
  dist_exact    ref-bf on sssp/ seeded from the source's own record (via hvmap)
  push_*        reference CPU forward_push (ref-push) pr / res on origin/ flist and on
                ppr/ wlist, for the listed sources and rmax values
The input graphs come from this library's seeded R-MAT writer, so the fixtures also
pin that generator's output.
"""
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "c-2graph_gb300"))

from oracle import build as obuild  # noqa: E402
import c2g  # noqa: E402

CASES = {
    # name: (scale, edge_factor, seed, wmax)
    "rmat_s10_ef8_seed3": (10, 8, 3, 100),
    "rmat_s12_ef8_seed5": (12, 8, 5, 1000),
}
NAMES = ("vlist", "elist", "wlist", "flist", "hvlist", "helist", "hwlist")


def tiny_case(d):
    """Hand-made 12-vertex graph: isolated vertices, a zero-in-degree hub, a chain,
    a triangle and low-in-degree vertices that the pruners remove edges from."""
    adj = {0: [(1, 4), (2, 1), (3, 7), (5, 2)], 1: [(2, 2), (4, 3)], 2: [(4, 1), (6, 9)],
           3: [(4, 2), (6, 1)], 4: [(5, 5), (7, 3)], 5: [(7, 1)], 6: [(7, 2), (8, 4)],
           7: [(8, 1)], 8: [(9, 6)], 9: [(7, 2)], 10: [], 11: []}
    V = 12
    vl, el, wl = [0], [], []
    for v in range(V):
        for t, w in sorted(adj[v]):
            el.append(t)
            wl.append(w)
        vl.append(len(el))
    vl, el, wl = (np.array(x, dtype=np.int32) for x in (vl, el, wl))
    fl = np.empty(len(el), dtype=np.float32)
    for v in range(V):
        s = wl[vl[v]:vl[v + 1]].sum()
        if vl[v + 1] > vl[v]:
            fl[vl[v]:vl[v + 1]] = (wl[vl[v]:vl[v + 1]] / s).astype(np.float32)
    for sub in ("origin", "sssp", "ppr"):
        os.makedirs(os.path.join(d, sub), exist_ok=True)
    for name, a in (("vlist", vl), ("elist", el), ("wlist", wl), ("flist", fl)):
        a.tofile(os.path.join(d, "origin", name + ".bin"))


def run(cmd):
    subprocess.run(cmd, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def read(d, sub, name, ppr=False):
    p = os.path.join(d, sub, name + ".bin")
    fl = name == "flist" or (ppr and name in ("wlist", "hwlist"))
    return np.fromfile(p, dtype=np.float32 if fl else np.int32) if os.path.exists(p) else None


def as_origin(src_dir, sub, dst, weights_float):
    """A dataset dir whose origin/ holds <src_dir>/<sub>/ so the reference harnesses
    (which read origin/) run on the pruned graph."""
    os.makedirs(os.path.join(dst, "origin"), exist_ok=True)
    for n in ("vlist", "elist"):
        shutil.copy(os.path.join(src_dir, sub, n + ".bin"), os.path.join(dst, "origin", n + ".bin"))
    shutil.copy(os.path.join(src_dir, sub, "wlist.bin"),
                os.path.join(dst, "origin", ("flist" if weights_float else "wlist") + ".bin"))


def ref_bf(d, s, seeds=None):
    with tempfile.TemporaryDirectory() as t:
        out = os.path.join(t, "d.bin")
        cmd = [obuild.ref_tool("ref-bf"), d, str(s), out]
        if seeds is not None:
            sp = os.path.join(t, "s.bin")
            np.asarray(seeds, dtype=np.int32).reshape(-1).tofile(sp)
            cmd.append(sp)
        run(cmd)
        return np.fromfile(out, dtype=np.int32)


def ref_push(d, s, rmax):
    with tempfile.TemporaryDirectory() as t:
        pre = os.path.join(t, "o")
        run([obuild.ref_tool("ref-push"), d, str(s), repr(float(np.float32(rmax))), pre])
        return np.fromfile(pre + ".pr.bin", dtype=np.float32), np.fromfile(pre + ".res.bin", dtype=np.float32)


def make(name, writer):
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        a, b = os.path.join(tmp, "ref"), os.path.join(tmp, "mine")
        writer(a)
        writer(b)
        run([obuild.ref_tool("purn-sssp"), a])
        run([obuild.ref_tool("purn-ppr"), a])
        c2g.prune_sssp(b)
        c2g.prune_ppr(b)
        for sub in ("sssp", "ppr"):
            for n in ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist"):
                ra, rb = read(a, sub, n, sub == "ppr"), read(b, sub, n, sub == "ppr")
                assert ra.tobytes() == rb.tobytes(), "pruner output differs: %s/%s" % (sub, n)
        for sub, names in (("origin", ("vlist", "elist", "wlist", "flist")), ("sssp", NAMES[:3] + NAMES[4:]),
                           ("ppr", NAMES[:3] + NAMES[4:])):
            for n in names:
                out["%s_%s" % (sub, n)] = read(a, sub, n, sub == "ppr")
        out["hvmap"] = read(b, "sssp", "hvmap")

        vl = out["origin_vlist"]
        V = len(vl) - 1
        deg = np.diff(vl)
        rng = np.random.default_rng(12345)
        cand = np.flatnonzero(deg > 0)
        srcs = [int(np.argmax(deg))] + [int(x) for x in rng.choice(cand, size=min(5, len(cand)), replace=False)]
        out["sources"] = np.array(srcs, dtype=np.int32)
        out["dist_origin"] = np.stack([ref_bf(a, s) for s in srcs])

        hv, he, hw = out["sssp_hvlist"], out["sssp_helist"], out["sssp_hwlist"]
        R = len(hv) - 1
        rec_of = np.full(V, -1, dtype=np.int64)
        rec_of[out["hvmap"]] = np.arange(R)
        pd = os.path.join(tmp, "pruned_sssp")
        as_origin(a, "sssp", pd, False)
        compat, exact = [], []
        for s in srcs:
            r = s if s < R else None
            seeds = None if r is None else np.stack([he[hv[r]:hv[r + 1]], hw[hv[r]:hv[r + 1]]], 1)
            compat.append(ref_bf(pd, s, seeds) if r is not None else np.full(V, -1, dtype=np.int32))
            r = rec_of[s]
            seeds = np.zeros((0, 2), np.int32) if r < 0 else np.stack([he[hv[r]:hv[r + 1]], hw[hv[r]:hv[r + 1]]], 1)
            exact.append(ref_bf(pd, s, seeds))
        out["dist_compat"] = np.stack(compat)
        out["dist_exact"] = np.stack(exact)

        rmaxes = [1e-3 / (V + 1), 1e-4]
        push_src = srcs[:2]
        pp = os.path.join(tmp, "pruned_ppr")
        as_origin(a, "ppr", pp, True)
        prs, ress, pprs, pres = [], [], [], []
        for s in push_src:
            for rm in rmaxes:
                p, r = ref_push(a, s, rm)
                prs.append(p)
                ress.append(r)
                p, r = ref_push(pp, s, rm)
                pprs.append(p)
                pres.append(r)
        out["push_sources"] = np.array(push_src, dtype=np.int32)
        out["push_rmax"] = np.array(rmaxes, dtype=np.float32)
        out["push_pr_origin"] = np.stack(prs)
        out["push_res_origin"] = np.stack(ress)
        out["push_pr_ppr"] = np.stack(pprs)
        out["push_res_ppr"] = np.stack(pres)
    path = os.path.join(HERE, name + ".npz")
    np.savez_compressed(path, **out)
    print("wrote", path, os.path.getsize(path), "bytes")


def main():
    if obuild.build_ref() is None:
        sys.exit("reference tree not found: cannot generate golden fixtures")
    obuild.build_oracle()
    for name, (scale, ef, seed, wmax) in CASES.items():
        make(name, lambda d, s=scale, e=ef, sd=seed, w=wmax: c2g.rmat_write(d, s, e, sd, 1, w))
    make("tiny12", tiny_case)


if __name__ == "__main__":
    main()
