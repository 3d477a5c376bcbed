"""SSSP on the GPU through the C ABI against the oracle: bit-exact int32 distances.

Golden cases: distances from the reference's own CPU Bellman-Ford (sssp-base
semantics on origin/, sssp-purn semantics on the reference-pruned sssp/ with
vertex-indexed seeds, and the exact-record mode).  Larger R-MAT graphs are checked
against the oracle's Dijkstra / seeded relaxation.
"""
import os
import re

import numpy as np
import pytest

from conftest import golden_cases, load_golden, write_dataset

pytestmark = pytest.mark.gpu

CONFIGS = [  # (delta, tile)
    (0, 256), (0, 32), (0, 4096), (40, 256), (500, 64), (3000, 1024)]


@pytest.fixture(scope="module")
def gdirs(tmp_path_factory, built):
    out = {}
    for name in golden_cases():
        g = load_golden(name)
        out[name] = (write_dataset(str(tmp_path_factory.mktemp(name)), g), g)
    return out


@pytest.fixture(scope="module")
def rmat16(tmp_path_factory, built):
    """R-MAT scale 16 / edge factor 16 / seed 1, weights in [1,100], pruned."""
    import c2g

    d = str(tmp_path_factory.mktemp("rmat16"))
    c2g.rmat_write(d, 16, 16, 1, 1, 100)
    c2g.prune_sssp(d)
    return d


def test_sssp_base_golden(gpu_available, gdirs):
    import c2g

    for name, (d, g) in gdirs.items():
        with c2g.Graph.load(d, "origin") as gr:
            for delta, tile in CONFIGS:
                gr.sssp_config(delta=delta, tile=tile)
                for s, ref in zip(g["sources"], g["dist_origin"]):
                    dist, st = gr.sssp(int(s))
                    assert np.array_equal(dist, ref), (name, s, delta, tile)
                    assert st.status_flags == 0


def test_sssp_purn_compat_golden(gpu_available, gdirs):
    import c2g

    for name, (d, g) in gdirs.items():
        with c2g.Graph.load(d, "sssp") as gr:
            R = len(g["sssp_hvlist"]) - 1
            for delta, tile in CONFIGS[:4]:
                gr.sssp_config(delta=delta, tile=tile)
                for s, ref in zip(g["sources"], g["dist_compat"]):
                    s = int(s)
                    if s >= R:
                        with pytest.raises(c2g.C2GError) as e:
                            gr.sssp(s, seeds=True, mode=c2g.SEEDS_COMPAT)
                        assert e.value.code == c2g.ERR_RANGE
                        continue
                    dist, _ = gr.sssp(s, seeds=True, mode=c2g.SEEDS_COMPAT)
                    assert np.array_equal(dist, ref), (name, s, delta, tile)


def test_sssp_purn_exact_golden(gpu_available, gdirs):
    import c2g

    for name, (d, g) in gdirs.items():
        with c2g.Graph.load(d, "sssp") as gr:
            for delta, tile in CONFIGS[:4]:
                gr.sssp_config(delta=delta, tile=tile)
                for s, ref in zip(g["sources"], g["dist_exact"]):
                    dist, _ = gr.sssp(int(s), seeds=True, mode=c2g.SEEDS_EXACT)
                    assert np.array_equal(dist, ref), (name, s, delta, tile)


def test_sssp_rmat16_vs_dijkstra(gpu_available, rmat16):
    """Config-1 graph: R-MAT s16/ef16/seed 1, source = highest out-degree vertex."""
    import c2g
    import oracle

    o = oracle.load_dataset(rmat16, "origin")
    deg = np.diff(o["vlist"])
    rng = np.random.default_rng(7)
    srcs = [int(np.argmax(deg))] + [int(x) for x in rng.choice(np.flatnonzero(deg > 0), 4, replace=False)]
    with c2g.Graph.load(rmat16, "origin") as gr:
        for delta, tile in CONFIGS:
            gr.sssp_config(delta=delta, tile=tile)
            for s in srcs:
                ref = oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [s], [0])
                dist, st = gr.sssp(s)
                assert np.array_equal(dist, ref), (s, delta, tile)
                reached = ref != oracle.INF_DIST
                assert st.edges_relaxed >= int(deg[reached].sum())


def test_sssp_rmat16_pruned_exact(gpu_available, rmat16):
    import c2g
    import oracle

    p = oracle.load_dataset(rmat16, "sssp")
    hv, he, hw, hvmap = p["hvlist"], p["helist"], p["hwlist"], p["hvmap"]
    rec_of = {int(v): r for r, v in enumerate(hvmap)}
    deg = np.diff(p["vlist"])
    srcs = [int(np.argmax(deg))] + [int(v) for v in hvmap[:3]]
    with c2g.Graph.load(rmat16, "sssp") as gr:
        for delta in (0, 200):
            gr.sssp_config(delta=delta)
            for s in srcs:
                r = rec_of.get(s)
                sv, sw = ((), ()) if r is None else (he[hv[r]:hv[r + 1]], hw[hv[r]:hv[r + 1]])
                ref, _ = oracle.sssp_seeded(p["vlist"], p["elist"], p["wlist"], s, sv, sw)
                dist, st = gr.sssp(s, seeds=True, mode=c2g.SEEDS_EXACT)
                assert np.array_equal(dist, ref), (s, delta)
                assert st.n_seeds == len(sv)


def test_sssp_edge_cases(gpu_available):
    import c2g

    # 0 -> 1 -> 2, 3 isolated, 4 -> 0 (never reached from 0), zero-weight edge 2 -> 5
    vl = np.array([0, 1, 2, 3, 3, 4, 4], np.int32)
    el = np.array([1, 2, 5, 0], np.int32)
    wl = np.array([7, 0, 0, 3], np.int32)
    with c2g.Graph.create(vl, el, wl) as gr:
        inf = c2g.INF_DIST
        for delta in (0, 1, 5):
            gr.sssp_config(delta=delta)
            d, _ = gr.sssp(0)
            assert d.tolist() == [0, 7, 7, inf, inf, 7]
            d, st = gr.sssp(3)  # no out-edges: only the source is reached
            assert d.tolist() == [inf, inf, inf, 0, inf, inf]
            assert st.vertices_popped == 0
            d, _ = gr.sssp(4)
            assert d.tolist() == [3, 10, 10, inf, 0, 10]
        with pytest.raises(c2g.C2GError) as e:
            gr.sssp(6)
        assert e.value.code == c2g.ERR_RANGE
        assert gr.resolve_source(3) == 4   # sssp-base skip rule: outdeg < 1 -> next
        with pytest.raises(c2g.C2GError):
            gr.resolve_source(5)
    # single vertex, no edges
    with c2g.Graph.create(np.array([0, 0], np.int32), np.zeros(0, np.int32), np.zeros(0, np.int32)) as gr:
        d, _ = gr.sssp(0)
        assert d.tolist() == [0]


def test_sssp_repeated_queries_share_workspace(gpu_available, rmat16):
    """Many queries on one handle (stamp epochs advance across launches), switching
    configurations in between."""
    import c2g
    import oracle

    o = oracle.load_dataset(rmat16, "origin")
    deg = np.diff(o["vlist"])
    rng = np.random.default_rng(3)
    srcs = rng.choice(np.flatnonzero(deg > 0), 24, replace=False)
    with c2g.Graph.load(rmat16, "origin") as gr:
        for i, s in enumerate(srcs):
            gr.sssp_config(delta=[0, 64, 700][i % 3], tile=[256, 128][i % 2])
            ref = oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [int(s)], [0])
            dist, _ = gr.sssp(int(s))
            assert np.array_equal(dist, ref), (i, s)


def test_sssp_device_output(gpu_available, rmat16):
    import torch

    import c2g
    import oracle

    o = oracle.load_dataset(rmat16, "origin")
    s = int(np.argmax(np.diff(o["vlist"])))
    with c2g.Graph.load(rmat16, "origin") as gr:
        out = torch.empty(gr.V, dtype=torch.int32, device="cuda:0")
        gr.sssp(s, out_ptr=out.data_ptr())
        host, _ = gr.sssp(s)
        assert np.array_equal(out.cpu().numpy(), host)


def test_sssp_iteration_cap(gpu_available, rmat16):
    """A round cap of 1 stops early: flagged, and distances are upper bounds."""
    import c2g
    import oracle

    o = oracle.load_dataset(rmat16, "origin")
    s = int(np.argmax(np.diff(o["vlist"])))
    ref = oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [s], [0])
    with c2g.Graph.load(rmat16, "origin") as gr:
        gr.sssp_config(delta=0, max_iter=1)
        d, st = gr.sssp(s)
        assert st.status_flags & c2g.FLAG_ITER_CAP
        assert np.all(d >= ref) and d[s] == 0
        gr.sssp_config(delta=0)
        d, st = gr.sssp(s)
        assert np.array_equal(d, ref) and st.status_flags == 0


def test_cli_sssp_base_output(gpu_available, gdirs):
    import subprocess

    from conftest import PKG

    d, g = gdirs["rmat_s10_ef8_seed3"]
    s = int(g["sources"][0])
    r = subprocess.run([os.path.join(PKG, "bin", "sssp-base"), d, str(s)], stdout=subprocess.PIPE, text=True,
                       check=True)
    lines = [l for l in r.stdout.splitlines() if re.fullmatch(r"\d+\t-?\d+", l)]
    vals = [int(l.split("\t")[1]) for l in lines[:10]]
    assert vals == g["dist_origin"][0][:10].tolist()
    assert "gpu runtime:" in r.stdout


def test_sssp_stress_mixed_configs(gpu_available, tmp_path_factory):
    """Many queries on one handle with weights in [1,1000] (the scale-22 distribution),
    cycling delta and tile sizes, each against Dijkstra: catches rare ordering races."""
    import c2g
    import oracle

    d = str(tmp_path_factory.mktemp("stress18"))
    c2g.rmat_write(d, 18, 16, 2, 1, 1000)
    o = oracle.load_dataset(d, "origin")
    deg = np.diff(o["vlist"])
    rng = np.random.default_rng(11)
    srcs = [int(np.argmax(deg))] + [int(x) for x in rng.choice(np.flatnonzero(deg > 0), 7, replace=False)]
    refs = {s: oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [s], [0]) for s in srcs}
    cfgs = [(0, 256), (25, 64), (25, 256), (100, 128), (400, 256), (1600, 1024), (0, 64), (50, 512)]
    with c2g.Graph.load(d, "origin") as gr:
        for rep in range(3):
            for i, (delta, tile) in enumerate(cfgs):
                gr.sssp_config(delta=delta, tile=tile)
                for s in srcs[(i + rep) % 4::2]:
                    dist, st = gr.sssp(s)
                    bad = int((dist != refs[s]).sum())
                    assert bad == 0, (rep, delta, tile, s, bad, int((dist > refs[s]).sum()))
                    assert st.status_flags == 0


def test_sssp_autotune(gpu_available, rmat16, tmp_path):
    import json

    import c2g
    import oracle

    o = oracle.load_dataset(rmat16, "origin")
    deg = np.diff(o["vlist"])
    srcs = [int(np.argmax(deg)), int(np.flatnonzero(deg > 0)[3])]
    with c2g.Graph.load(rmat16, "origin") as gr:
        path = str(tmp_path / "tune.json")
        delta, tile = gr.sssp_autotune(srcs, json_path=path)
        rec = json.load(open(path))
        assert rec["best"]["delta"] == delta and rec["best"]["tile"] == tile
        assert all(c["valid"] for c in rec["candidates"])
        assert len(rec["candidates"]) == 40
        ref = oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [srcs[0]], [0])
        d, _ = gr.sssp(srcs[0])  # the tuned configuration is applied
        assert np.array_equal(d, ref)


def test_watchdog_barrier_timeout_is_reported_and_recoverable(gpu_available, rmat16):
    """Failure detection without a fault: the next launch's grid barrier waits for one
    block more than the grid has, every bounded wait runs out after 100 ms, the call
    returns C2G_ERR_TIMEOUT, and the same handle answers the next query correctly."""
    import time

    import c2g
    import oracle

    o = oracle.load_dataset(rmat16, "origin")
    deg = np.diff(o["vlist"])
    s = int(np.argmax(deg))
    with c2g.Graph.load(rmat16, "origin") as g:
        g.watchdog(barrier_timeout_ms=100, stall_next_sssp=True)
        t0 = time.time()
        with pytest.raises(c2g.C2GError) as ei:
            g.sssp(s)
        assert ei.value.code == -7  # C2G_ERR_TIMEOUT
        assert time.time() - t0 < 10.0
        g.watchdog()  # default limits again
        dist, st = g.sssp(s)
        assert st.status_flags == 0
        ref = oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [s], [0])
        assert np.array_equal(dist, ref)
