"""Serving loop: continuous batching with the graph resident on the device.  Requests
arrive while others run, join the running SSSP / PPR batches at the next epoch, and
each result must be the same as the query run alone: SSSP bit-exact against the
oracle's Dijkstra, PPR within L1 1e-6 of the FP64 push, adsorption within 1e-6 (max) of
the single call, which its own test checks against the FP64 recurrence."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _check_results(g, o, pp, results):
    import c2g
    import oracle

    for kind, s, seeds, out in results:
        if kind == c2g.REQ_SSSP:
            assert np.array_equal(out, oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [s], [0])), s
        elif kind == c2g.REQ_PPR:
            rp, _, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], s, 0.15, 1e-7)
            assert float(np.abs(out.astype(np.float64) - rp).sum()) <= 1e-6, s
        else:
            alone, _ = g.adsorption(seeds, pp[:, 0], pp[:, 1], pp[:, 2], 30)
            assert float(np.abs(out.astype(np.float64) - alone).max()) <= 1e-6


def test_server_mix_equals_alone(gpu_available, tmp_path):
    """Three waves of requests, each submitted while the previous ones are on the device;
    every result equals the query alone, and later requests joined running batches (the
    SSSP and PPR batches ran more epochs than there were waves)."""
    import c2g
    import oracle

    d = str(tmp_path / "g")
    c2g.rmat_write(d, 14, 16, 8, 1, 1000)
    o = oracle.load_dataset(d, "origin")
    V = len(o["vlist"]) - 1
    rng = np.random.default_rng(5)
    pp = rng.dirichlet((1.0, 1.0, 1.0), size=V).astype(np.float32)
    cand = np.flatnonzero(np.diff(o["vlist"]) > 0)
    kinds = [c2g.REQ_SSSP] * 42 + [c2g.REQ_PPR] * 21 + [c2g.REQ_ADSORPTION] * 6
    rng.shuffle(kinds)
    subs = []
    with c2g.Graph.load(d, "origin") as g:
        with c2g.Server(g, max_batch=32, alpha=0.15, rmax=1e-7, ads_iterations=30, p_inj=pp[:, 0], p_cont=pp[:, 1],
                        p_abnd=pp[:, 2], epoch_rounds=2) as srv:
            for wave in range(3):
                for k in kinds[wave::3]:
                    if k == c2g.REQ_ADSORPTION:
                        out, s = np.empty((V, 16), np.float32), 0
                        seeds = rng.choice(V, 16, replace=False).astype(np.int32)
                    else:
                        out = np.empty(V, np.int32 if k == c2g.REQ_SSSP else np.float32)
                        s, seeds = int(rng.choice(cand)), None
                    subs.append((srv.submit(k, source=s, seeds=seeds, out=out), k, s, seeds, out))
                time.sleep(0.02)
            results = []
            for t, k, s, seeds, out in subs:
                st, ms = srv.wait(t)
                assert st == 0 and ms > 0
                results.append((k, s, seeds, out))
            stats = srv.stats()
        assert stats.completed == len(subs)
        assert stats.p50_ms > 0 and stats.p99_ms >= stats.p50_ms
        assert stats.max_batch > 1  # queries ran together
        assert stats.batches[0] > 3 and stats.batches[1] > 3  # epochs, with joins between them
        _check_results(g, o, pp, results)


def test_server_results_match_single_calls(gpu_available, tmp_path):
    """Two client threads submit at once into small batches (8 slots), so requests wait
    for slots and join as others finish."""
    import c2g
    import oracle

    d = str(tmp_path / "g")
    c2g.rmat_write(d, 13, 16, 9, 1, 1000)
    o = oracle.load_dataset(d, "origin")
    V = len(o["vlist"]) - 1
    rng = np.random.default_rng(9)
    pp = rng.dirichlet((1.0, 1.0, 1.0), size=V).astype(np.float32)
    cand = np.flatnonzero(np.diff(o["vlist"]) > 0)
    work = [(c2g.REQ_SSSP, int(rng.choice(cand)), None) for _ in range(30)]
    work += [(c2g.REQ_PPR, int(rng.choice(cand)), None) for _ in range(12)]
    work += [(c2g.REQ_ADSORPTION, 0, rng.choice(V, 16, replace=False).astype(np.int32)) for _ in range(4)]
    with c2g.Graph.load(d, "origin") as g:
        with c2g.Server(g, max_batch=8, alpha=0.15, rmax=1e-7, ads_iterations=30, p_inj=pp[:, 0], p_cont=pp[:, 1],
                        p_abnd=pp[:, 2], epoch_rounds=3) as srv:
            tickets = []
            lock = threading.Lock()

            def client(items):
                for kind, s, seeds in items:
                    if kind == c2g.REQ_ADSORPTION:
                        out = np.empty((V, 16), np.float32)
                    else:
                        out = np.empty(V, np.int32 if kind == c2g.REQ_SSSP else np.float32)
                    t = srv.submit(kind, source=s, seeds=seeds, out=out)
                    with lock:
                        tickets.append((t, kind, s, seeds, out))

            th = [threading.Thread(target=client, args=(work[i::2],)) for i in range(2)]
            for x in th:
                x.start()
            for x in th:
                x.join()
            results = []
            for t, kind, s, seeds, out in tickets:
                st, _ = srv.wait(t)
                assert st == 0
                results.append((kind, s, seeds, out))
            stats = srv.stats()
        assert stats.completed == len(work) and stats.max_batch <= 8 + 8
        _check_results(g, o, pp, results)


def test_server_preemption_keeps_results(gpu_available, tmp_path):
    """With 4 slots per kind and preemption after 2 rounds, waiting requests evict the
    longest-running queries into snapshots; the evicted queries resume and finish with
    the results they would have had alone."""
    import c2g
    import oracle

    d = str(tmp_path / "g")
    c2g.rmat_write(d, 14, 16, 10, 1, 1000)
    o = oracle.load_dataset(d, "origin")
    V = len(o["vlist"]) - 1
    rng = np.random.default_rng(12)
    cand = np.flatnonzero(np.diff(o["vlist"]) > 0)
    work = [(c2g.REQ_SSSP, int(s)) for s in rng.choice(cand, 16, replace=False)]
    work += [(c2g.REQ_PPR, int(s)) for s in rng.choice(cand, 12, replace=False)]
    rng.shuffle(work)
    with c2g.Graph.load(d, "origin") as g:
        with c2g.Server(g, max_batch=4, alpha=0.15, rmax=1e-7, epoch_rounds=1, preempt_rounds=2) as srv:
            subs = []
            for k, s in work:
                out = np.empty(V, np.int32 if k == c2g.REQ_SSSP else np.float32)
                subs.append((srv.submit(k, source=s, out=out), k, s, out))
                time.sleep(0.002)
            results = []
            for t, k, s, out in subs:
                st, _ = srv.wait(t)
                assert st == 0
                results.append((k, s, None, out))
            stats = srv.stats()
        assert stats.evictions > 0
        _check_results(g, o, None, results)
