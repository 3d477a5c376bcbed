"""Batched multi-tenant SSSP (one persistent launch, per-query bitmask frontiers)
against the per-source oracle: every query's distances bit-exact."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def g16(tmp_path_factory, built):
    import c2g

    d = str(tmp_path_factory.mktemp("b16"))
    c2g.rmat_write(d, 16, 16, 1, 1, 100)
    c2g.prune_sssp(d)
    return d


@pytest.fixture(scope="module")
def g17w(tmp_path_factory, built):
    import c2g

    d = str(tmp_path_factory.mktemp("b17"))
    c2g.rmat_write(d, 17, 16, 2, 1, 1000)
    return d


def _sources(vl, n, seed):
    deg = np.diff(vl)
    rng = np.random.default_rng(seed)
    top = np.argsort(-deg, kind="stable")[: max(1, len(deg) // 100)]
    s = list(rng.choice(np.flatnonzero(deg > 0), n - n // 2, replace=False)) + list(rng.choice(top, n // 2))
    return np.array(s, dtype=np.int32)


@pytest.mark.parametrize("n", [1, 31, 40, 64, 100])
def test_batch_vs_dijkstra(gpu_available, g17w, n):
    import c2g
    import oracle

    o = oracle.load_dataset(g17w, "origin")
    src = _sources(o["vlist"], n, n)
    src[-1] = src[0]  # a repeated source
    with c2g.Graph.load(g17w, "origin") as gr:
        dist, st = gr.sssp_batch(src)
        assert st.status_flags == 0
        assert dist.shape == (n, gr.V)
        for i, s in enumerate(src):
            ref = oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [int(s)], [0])
            assert np.array_equal(dist[i], ref), (n, i, s)


@pytest.mark.parametrize("frac", [-1.0, 0.0, 0.5])
def test_sssp_batch_pull_shapes_vs_dijkstra(gpu_available, g17w, g16, frac):
    """Expand-only rounds, pull rounds in every round and the default mix give the exact
    distances: 1, 2, 4 and 8 query words on origin/ (float and int weights, so the pull's
    int32 in-edges are a second scatter), and EXACT-seeded queries on the pruned sssp/
    (int weights only: the pull uses the one reverse CSR) against the single query."""
    import c2g
    import oracle

    o = oracle.load_dataset(g17w, "origin")
    with c2g.Graph.load(g17w, "origin") as gr:
        gr.sssp_batch_pull(frac)
        for n in (20, 50, 100, 256):
            src = _sources(o["vlist"], n, 40 + n)
            dist, st = gr.sssp_batch(src)
            assert st.status_flags == 0
            for i in range(0, n, max(1, n // 16)):  # a sample of the queries
                ref = oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [int(src[i])], [0])
                assert np.array_equal(dist[i], ref), (frac, n, i)
    with c2g.Graph.load(g16, "sssp") as gr:
        gr.sssp_batch_pull(frac)
        vl = np.fromfile(g16 + "/sssp/vlist.bin", dtype=np.int32)
        src = _sources(vl, 96, 7)
        dist, st = gr.sssp_batch(src, seeds=True, mode=c2g.SEEDS_EXACT)
        assert st.status_flags == 0
        for i in range(0, 96, 6):
            ref, _ = gr.sssp(int(src[i]), seeds=True, mode=c2g.SEEDS_EXACT)
            assert np.array_equal(dist[i], ref), (frac, i)


def test_batch_tiles_and_autotune(gpu_available, g17w, tmp_path):
    """Every tile shape gives the same distances (Dijkstra); the autotuner times its 13 tile
    candidates, then 4 more pull fractions at the fastest tiles, keeps valid ones and
    applies them."""
    import json

    import c2g
    import oracle

    o = oracle.load_dataset(g17w, "origin")
    src = _sources(o["vlist"], 96, 5)
    refs = [oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [int(s)], [0]) for s in src[:6]]
    with c2g.Graph.load(g17w, "origin") as gr:
        for big, mn in ((128, 1), (256, 1), (1024, 4), (4096, 1024)):
            gr.sssp_batch_tile(big, mn)
            dist, st = gr.sssp_batch(src)
            assert st.status_flags == 0
            for i in range(6):
                assert np.array_equal(dist[i], refs[i]), (big, mn, i)
        with pytest.raises(c2g.C2GError):
            gr.sssp_batch_tile(100, 4)
        with pytest.raises(c2g.C2GError):
            gr.sssp_batch_tile(512, 3)
        path = str(tmp_path / "tile.json")
        big, mn = gr.sssp_batch_autotune(src, reps=1, json_path=path)
        rec = json.load(open(path))
        assert len(rec["candidates"]) == 17 and all(c["valid"] for c in rec["candidates"])
        assert (rec["best"]["big_steps"], rec["best"]["min_tiles_per_warp"]) == (big, mn)
        assert {c["pull_frac"] for c in rec["candidates"][13:]} | {0.3} == {-1, 0.15, 0.3, 0.5, 0.75}
        b = ctypes_tile(gr)
        assert b == (big, mn)
        assert abs(gr.sssp_batch_pull_frac() - rec["best"]["pull_frac"]) < 1e-6
        dist, _ = gr.sssp_batch(src)
        for i in range(6):
            assert np.array_equal(dist[i], refs[i])


def ctypes_tile(gr):
    import ctypes

    import c2g

    b, m = ctypes.c_int32(), ctypes.c_int32()
    assert c2g.lib().c2g_sssp_batch_get_tile(gr._h, ctypes.byref(b), ctypes.byref(m)) == 0
    return b.value, m.value


def test_batch_matches_single_query_with_seeds(gpu_available, g16):
    import c2g

    with c2g.Graph.load(g16, "sssp") as gr:
        hvmap = np.fromfile(g16 + "/sssp/hvmap.bin", dtype=np.int32)
        vl = np.fromfile(g16 + "/sssp/vlist.bin", dtype=np.int32)
        deg = np.diff(vl)
        src = np.concatenate([hvmap[:20], _sources(vl, 20, 3)]).astype(np.int32)
        src = src[deg[src] >= 0]
        for mode in (c2g.SEEDS_EXACT, c2g.SEEDS_COMPAT):
            s_ok = src if mode == c2g.SEEDS_EXACT else src[src < gr.R]
            dist, st = gr.sssp_batch(s_ok, seeds=True, mode=mode)
            for i, s in enumerate(s_ok):
                ref, _ = gr.sssp(int(s), seeds=True, mode=mode)
                assert np.array_equal(dist[i], ref), (mode, i, s)


def test_batch_layouts_and_device_output(gpu_available, g16):
    import torch

    import c2g

    with c2g.Graph.load(g16, "origin") as gr:
        src = _sources(np.fromfile(g16 + "/origin/vlist.bin", dtype=np.int32), 48, 5)
        qm, _ = gr.sssp_batch(src)
        vm, _ = gr.sssp_batch(src, vertex_major=True)
        assert np.array_equal(qm, vm.T)
        out = torch.empty((len(src), gr.V), dtype=torch.int32, device="cuda:0")
        gr.sssp_batch(src, out_ptr=out.data_ptr())
        assert np.array_equal(out.cpu().numpy(), qm)
        # single-query path agrees too
        for i in (0, 17, 47):
            ref, _ = gr.sssp(int(src[i]))
            assert np.array_equal(qm[i], ref)


def test_batch_rejects_bad_sources(gpu_available, g16):
    import c2g

    with c2g.Graph.load(g16, "origin") as gr:
        with pytest.raises(c2g.C2GError) as e:
            gr.sssp_batch(np.array([0, gr.V], np.int32))
        assert e.value.code == c2g.ERR_RANGE


@pytest.fixture(scope="module")
def g14p(tmp_path_factory, built):
    import c2g

    d = str(tmp_path_factory.mktemp("pb14"))
    c2g.rmat_write(d, 14, 16, 2, 1, 1000)
    c2g.prune_ppr(d)
    return d


def _l1(a, b):
    return float(np.abs(a.astype(np.float64) - b).sum())


@pytest.mark.parametrize("n", [1, 33, 70])
def test_ppr_batch_base_vs_fp64(gpu_available, g14p, n):
    """Batched push, base init: each query within L1 <= 1e-6 of the FP64 oracle."""
    import c2g
    import oracle

    o = oracle.load_dataset(g14p, "origin")
    src = _sources(o["vlist"], n, 100 + n)
    with c2g.Graph.load(g14p, "origin") as gr:
        prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0, max_iter=500)
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags == 0 and pr.shape == (n, gr.V)
        for i, s in enumerate(src):
            rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(s), 0.15, 1e-7)
            assert _l1(pr[i], rp) <= 1e-6, (i, s, _l1(pr[i], rp))
            assert _l1(res[i], rr) <= 1e-6


def test_ppr_batch_seeded_pruned_vs_fp64(gpu_available, g14p):
    import c2g
    import oracle

    p = oracle.load_dataset(g14p, "ppr")
    hv, he, hw = p["hvlist"], p["helist"], p["hwlist"]
    src = np.concatenate([np.flatnonzero(np.diff(hv) > 0)[:10], _sources(p["vlist"], 22, 9)]).astype(np.int32)
    with c2g.Graph.load(g14p, "ppr") as gr:
        prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=1)
        pr, res, st = gr.ppr_batch(src, prm)
        for i, s in enumerate(src):
            s = int(s)
            sv = np.concatenate([he[hv[s]:hv[s + 1]], p["elist"][p["vlist"][s]:p["vlist"][s + 1]]])
            sw = np.concatenate([hw[hv[s]:hv[s + 1]], p["wlist"][p["vlist"][s]:p["vlist"][s + 1]]])
            rp, rr, _, _ = oracle.ppr_push(p["vlist"], p["elist"], p["wlist"], s, 0.15, 1e-7, seeded=True,
                                           seed_v=sv, seed_w=sw)
            assert _l1(pr[i], rp) <= 1e-6, (i, s)
            assert _l1(res[i], rr) <= 1e-6


def test_ppr_batch_matches_single_and_cap(gpu_available, g14p):
    import c2g
    import oracle

    o = oracle.load_dataset(g14p, "origin")
    src = _sources(o["vlist"], 40, 77)
    with c2g.Graph.load(g14p, "origin") as gr:
        prm = gr.ppr_params(alpha=0.2, rmax=1e-6, seeded=0, pr0=0.2, r0=1.0)
        pr, res, _ = gr.ppr_batch(src, prm, vertex_major=True)
        for i in (0, 13, 39):
            p1, r1, _ = gr.ppr(int(src[i]), prm)
            assert _l1(pr[:, i], p1.astype(np.float64)) <= 2e-6
        prm.max_iter = 3
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags & c2g.FLAG_ITER_CAP
        for i in (0, 21):
            rp, rr, rounds, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(src[i]), 0.2, 1e-6,
                                                max_iter=3)
            assert _l1(pr[i], rp) <= 1e-6 and _l1(res[i], rr) <= 1e-6


@pytest.mark.parametrize("ratio", [-1.0, 0.0, 8.0])
def test_ppr_batch_pull_shapes_vs_fp64(gpu_available, g14p, ratio):
    """Push-only, pull-every-round and the default mix: every query within L1 <= 1e-6 of
    the FP64 oracle, base and seeded, with the pushes counted the same way."""
    import c2g
    import oracle

    o = oracle.load_dataset(g14p, "origin")
    src = _sources(o["vlist"], 48, 5)
    with c2g.Graph.load(g14p, "origin") as gr:
        gr.ppr_batch_pull(ratio)
        prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0, max_iter=500)
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags == 0
        for i in (0, 7, 23, 24, 40, 47):
            rp, rr, _, cnt = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(src[i]), 0.15, 1e-7)
            assert _l1(pr[i], rp) <= 1e-6, (ratio, i, _l1(pr[i], rp))
            assert _l1(res[i], rr) <= 1e-6, (ratio, i, _l1(res[i], rr))
    p = oracle.load_dataset(g14p, "ppr")
    hv, he, hw = p["hvlist"], p["helist"], p["hwlist"]
    src = _sources(p["vlist"], 40, 6)
    with c2g.Graph.load(g14p, "ppr") as gr:
        gr.ppr_batch_pull(ratio)
        prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=1)
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags == 0
        for i in (0, 19, 20, 39):
            s = int(src[i])
            sv = np.concatenate([he[hv[s]:hv[s + 1]], p["elist"][p["vlist"][s]:p["vlist"][s + 1]]])
            sw = np.concatenate([hw[hv[s]:hv[s + 1]], p["wlist"][p["vlist"][s]:p["vlist"][s + 1]]])
            rp, rr, _, _ = oracle.ppr_push(p["vlist"], p["elist"], p["wlist"], s, 0.15, 1e-7, seeded=True,
                                           seed_v=sv, seed_w=sw)
            assert _l1(pr[i], rp) <= 1e-6, (ratio, i)
            assert _l1(res[i], rr) <= 1e-6, (ratio, i)


def test_ppr_batch_pull_cap_and_heavy_weights(gpu_available, g14p):
    """Pull every round: a round cap keeps the activated residuals; weights whose
    out-sums exceed 1 (the residual grows) narrow the fixed-point range and still match
    the FP64 oracle."""
    import c2g
    import oracle

    o = oracle.load_dataset(g14p, "origin")
    src = _sources(o["vlist"], 36, 8)
    with c2g.Graph.load(g14p, "origin") as gr:
        gr.ppr_batch_pull(0.0)
        prm = gr.ppr_params(alpha=0.2, rmax=1e-6, seeded=0, pr0=0.2, r0=1.0, max_iter=4)
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags & c2g.FLAG_ITER_CAP
        for i in (0, 35):
            rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(src[i]), 0.2, 1e-6, max_iter=4)
            assert _l1(pr[i], rp) <= 1e-6 and _l1(res[i], rr) <= 1e-6
        # a second launch after the cap starts from clean state
        prm.max_iter = 500
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags == 0
        rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(src[3]), 0.2, 1e-6)
        assert _l1(pr[3], rp) <= 1e-6 and _l1(res[3], rr) <= 1e-6
        heavy = (o["flist"].astype(np.float32) * np.float32(3.0)).astype(np.float32)
        gr.set_weights(heavy)
        prm = gr.ppr_params(alpha=0.2, rmax=1e-6, seeded=0, pr0=0.2, r0=1.0, max_iter=6)
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags == c2g.FLAG_ITER_CAP or st.status_flags == 0
        for i in (1, 30):
            rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], heavy, int(src[i]), 0.2, 1e-6, max_iter=6)
            scale = max(1.0, float(np.abs(rp).sum()))
            assert _l1(pr[i], rp) <= 1e-6 * scale, (i, _l1(pr[i], rp), scale)
            assert _l1(res[i], rr) <= 1e-6 * max(1.0, float(np.abs(rr).sum())), i


def test_batch_outputs_into_pinned_host_memory(gpu_available, g16):
    """Page-locked host outputs are written by the kernels directly; pageable ones go
    through a device stage and a copy.  Both give the same arrays, in both layouts."""
    import ctypes

    import torch

    import c2g

    with c2g.Graph.load(g16, "origin") as gr:
        src = _sources(np.fromfile(g16 + "/origin/vlist.bin", dtype=np.int32), 45, 21)
        for vm in (False, True):
            ref, _ = gr.sssp_batch(src, vertex_major=vm)
            pinned = torch.empty(ref.shape, dtype=torch.int32).pin_memory().numpy()
            pinned.fill(-7)
            got, st = gr.sssp_batch(src, out=pinned, vertex_major=vm)
            assert st.status_flags == 0 and np.array_equal(pinned, ref), vm
        prm = gr.ppr_params(alpha=0.15, rmax=1e-6, seeded=0, pr0=0.15, r0=1.0)
        pr_ref, _, _ = gr.ppr_batch(src, prm, want_res=False)
        pinned = torch.empty(pr_ref.shape, dtype=torch.float32).pin_memory().numpy()
        pinned.fill(-1.0)
        st = c2g.Stats()
        s = np.ascontiguousarray(src, dtype=np.int32)
        c2g._check(c2g.lib().c2g_ppr_batch(gr._h, len(s), c2g._ptr(s), ctypes.byref(prm), c2g._ptr(pinned), None,
                                           0, 0, ctypes.byref(st)))
        assert st.status_flags == 0
        assert np.abs(pinned.astype(np.float64) - pr_ref).sum(axis=1).max() <= 1e-9


def test_ppr_batch_autotune(gpu_available, g14p, tmp_path):
    """The pull-ratio autotuner times its candidates on the batch, records them, applies
    a valid one, and the batch under it still matches the FP64 oracle."""
    import json

    import c2g
    import oracle

    o = oracle.load_dataset(g14p, "origin")
    src = _sources(o["vlist"], 64, 12)
    path = str(tmp_path / "pull.json")
    with c2g.Graph.load(g14p, "origin") as gr:
        prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)
        best = gr.ppr_batch_autotune(src, prm, reps=1, json_path=path)
        rec = json.load(open(path))
        assert len(rec["candidates"]) == 7 and rec["candidates"][0]["ratio"] == -1
        assert rec["best"]["ratio"] == best and any(c["ratio"] == best and c["valid"] for c in rec["candidates"])
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags == 0
        rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(src[5]), 0.15, 1e-7)
        assert _l1(pr[5], rp) <= 1e-6 and _l1(res[5], rr) <= 1e-6


@pytest.mark.parametrize("n", [20, 100, 200])
def test_ppr_batch_pull_word_counts_vs_fp64(gpu_available, g14p, n):
    """Pull every round with 1, 4 and 8 query words per vertex (scalar and vector mask
    loads, one or two word groups per tile): each checked query within L1 <= 1e-6 of the
    FP64 oracle."""
    import c2g
    import oracle

    o = oracle.load_dataset(g14p, "origin")
    src = _sources(o["vlist"], n, 300 + n)
    with c2g.Graph.load(g14p, "origin") as gr:
        gr.ppr_batch_pull(0.0)
        prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)
        pr, res, st = gr.ppr_batch(src, prm)
        assert st.status_flags == 0
        for i in sorted({0, n // 3, n // 2, n - 1}):
            rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(src[i]), 0.15, 1e-7)
            assert _l1(pr[i], rp) <= 1e-6, (n, i, _l1(pr[i], rp))
            assert _l1(res[i], rr) <= 1e-6, (n, i)


def test_batch_round_trace(gpu_available, g17w, g14p):
    """The per-round trace of a batched launch: one entry per round, the work units add
    up to the launch's counters, and the rounds' times add up to (nearly all of) the
    launch's device time."""
    import c2g

    with c2g.Graph.load(g17w, "origin") as gr:
        src = _sources(np.fromfile(g17w + "/origin/vlist.bin", dtype=np.int32), 64, 4)
        for frac, want in ((-1.0, 0), (0.0, 1), (0.5, None)):
            gr.sssp_batch_pull(frac)
            _, st = gr.sssp_batch(src)
            ms, work, shape = gr.last_rounds()
            assert len(ms) == st.iterations and len(ms) > 3
            assert int(work.sum()) == st.touched  # edge-word steps
            if want is not None:  # expand only / pull every round
                assert np.all(shape == want), frac
            assert np.all(ms > 0)
            assert 0.5 * st.device_ms <= ms.sum() <= st.device_ms * 1.01
    with c2g.Graph.load(g14p, "origin") as gr:
        vl = np.fromfile(g14p + "/origin/vlist.bin", dtype=np.int32)
        src = _sources(vl, 64, 6)
        prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)
        gr.ppr_batch_pull(1.0)
        _, _, st = gr.ppr_batch(src, prm, want_res=False)
        ms, first, work, shape = gr.last_rounds(first_phase=True)
        assert len(ms) == st.iterations
        assert np.all(first > 0) and np.all(first < ms)  # the apply sweep follows the push / pull
        assert int(work.sum()) == st.edges_relaxed  # (query, edge) pushes
        assert shape.max() == 1 and shape.min() == 0  # some rounds pulled, some pushed
        assert 0.5 * st.device_ms <= ms.sum() <= st.device_ms * 1.01
