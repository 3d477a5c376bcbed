"""Resident batches (c2g_session_*): queries admitted while others run join at the next
epoch, finished slots are reused, and a query evicted into a snapshot and resumed (in the
same or another session) continues the same rounds.  Every result is checked against the
oracle: SSSP bit-exact (Dijkstra), PPR within L1 1e-6 of the FP64 push on pr and res."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
L1_TOL = 1e-6


@pytest.fixture(scope="module")
def g15(tmp_path_factory, built):
    import c2g

    d = str(tmp_path_factory.mktemp("sess15"))
    c2g.rmat_write(d, 15, 16, 6, 1, 1000)
    return d


def _srcs(vl, n, seed):
    deg = np.diff(vl)
    rng = np.random.default_rng(seed)
    top = np.argsort(-deg, kind="stable")[:64]
    return [int(x) for x in rng.choice(np.flatnonzero(deg > 0), n - n // 4, replace=False)] + \
        [int(x) for x in rng.choice(top, n // 4, replace=False)]


def _run(sess, plan, rounds, on_done):
    """Sources arrive at the epochs `plan` lists ({epoch: [sources]}) and wait for a free
    slot; step until every query finished; on_done(source, slot) reads each finished
    slot (which frees it)."""
    import c2g

    slot_src = {}
    epoch = 0
    arriving = {e: list(v) for e, v in plan.items()}
    queue = []
    while True:
        queue += arriving.pop(epoch, [])
        while queue:
            try:
                slot_src[sess.admit(queue[0])] = queue[0]
            except c2g.C2GError as e:
                assert e.code == c2g.ERR_OVERFLOW  # every slot taken: wait for one
                break
            queue.pop(0)
        fin, st = sess.step(rounds)
        assert st.status_flags == 0
        for sl in fin:
            on_done(slot_src.pop(sl), sl)
        epoch += 1
        if not slot_src and not arriving and not queue:
            return epoch
        assert epoch < 2000, "queries did not finish"


def test_session_sssp_staggered_admission_and_slot_reuse(gpu_available, g15):
    import c2g
    import oracle

    o = oracle.load_dataset(g15, "origin")
    srcs = _srcs(o["vlist"], 80, 1)
    plan = {0: srcs[:24], 1: srcs[24:40], 3: srcs[40:56], 6: srcs[56:]}
    seen = []
    with c2g.Graph.load(g15, "origin") as g, c2g.Session(g, c2g.REQ_SSSP, 48) as sess:
        def done(s, sl):
            dist, st = sess.read(sl)
            assert st.source == s
            assert np.array_equal(dist, oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [s], [0])), s
            seen.append(s)

        _run(sess, plan, 3, done)
    assert sorted(seen) == sorted(srcs)  # 80 queries through 48 slots: slots were reused


@pytest.mark.parametrize("frac", [0.0, -1.0])
def test_session_sssp_pull_rounds(gpu_available, g15, frac):
    """Resident SSSP batches whose rounds all pull over the reverse CSR (frac 0: every
    round with a frontier pulls) or all expand (frac -1): queries joining at epoch
    boundaries still get the exact distances, so the pull lookups rebuilt by each epoch's
    sweeps hold no stale state."""
    import c2g
    import oracle

    o = oracle.load_dataset(g15, "origin")
    srcs = _srcs(o["vlist"], 40, 11)
    plan = {0: srcs[:12], 1: srcs[12:24], 4: srcs[24:]}
    seen = []
    with c2g.Graph.load(g15, "origin") as g:
        g.sssp_batch_pull(frac)
        with c2g.Session(g, c2g.REQ_SSSP, 32) as sess:
            def done(s, sl):
                dist, st = sess.read(sl)
                assert np.array_equal(dist, oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [s], [0])), (frac, s)
                seen.append(s)

            _run(sess, plan, 2, done)
    assert sorted(seen) == sorted(srcs)


def test_session_ppr_staggered_admission_vs_fp64(gpu_available, g15):
    import c2g
    import oracle

    o = oracle.load_dataset(g15, "origin")
    srcs = _srcs(o["vlist"], 40, 2)
    plan = {0: srcs[:16], 2: srcs[16:28], 5: srcs[28:]}
    seen = []
    with c2g.Graph.load(g15, "origin") as g:
        prm = g.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0, max_iter=500)
        with c2g.Session(g, c2g.REQ_PPR, 32, prm) as sess:
            def done(s, sl):
                (pr, res), st = sess.read(sl, want_res=True)
                rp, rr, rounds, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], s, 0.15, 1e-7)
                assert float(np.abs(pr.astype(np.float64) - rp).sum()) <= L1_TOL, s
                assert float(np.abs(res.astype(np.float64) - rr).sum()) <= L1_TOL, s
                assert abs(st.iterations - rounds) <= 4 and st.status_flags == 0
                seen.append(s)

            _run(sess, plan, 4, done)
    assert sorted(seen) == sorted(srcs)


@pytest.mark.parametrize("kind", ["sssp", "ppr"])
def test_session_evict_and_resume(gpu_available, g15, kind):
    """Evict running queries after a few epochs, let the others run on, resume the
    snapshots (two in the same session, one in a second session on the same graph) and
    finish: the results are those of queries never interrupted."""
    import c2g
    import oracle

    o = oracle.load_dataset(g15, "origin")
    srcs = _srcs(o["vlist"], 12, 3)
    k = c2g.REQ_SSSP if kind == "sssp" else c2g.REQ_PPR
    with c2g.Graph.load(g15, "origin") as g:
        prm = g.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0, max_iter=500) if k else None
        results = {}

        def check(s, out):
            if k == c2g.REQ_SSSP:
                assert np.array_equal(out, oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [s], [0])), s
            else:
                rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], s, 0.15, 1e-7)
                assert float(np.abs(out[0].astype(np.float64) - rp).sum()) <= L1_TOL, s
                assert float(np.abs(out[1].astype(np.float64) - rr).sum()) <= L1_TOL, s
            results[s] = True

        with c2g.Session(g, k, 32, prm) as a, c2g.Session(g, k, 32, prm) as b:
            slot_src = {a.admit(s): s for s in srcs}
            for _ in range(2):
                fin, _ = a.step(1)
                for sl in fin:
                    out, _ = a.read(sl, want_res=True) if k else a.read(sl)
                    check(slot_src.pop(sl), out)
            victims = [sl for sl in list(slot_src)[:3]]
            assert len(victims) == 3, "queries finished too early for the test"
            snaps = [(slot_src.pop(sl), a.evict(sl)) for sl in victims]
            for sl in victims:
                assert a.slot(sl)[0] == 0  # freed at once
            for _ in range(3):  # the others run on without them
                fin, _ = a.step(2)
                for sl in fin:
                    out, _ = a.read(sl, want_res=True) if k else a.read(sl)
                    check(slot_src.pop(sl), out)
            where = {}
            for i, (s, snap) in enumerate(snaps):
                sess = b if i == 2 else a
                where[(sess is b, sess.resume(snap))] = s
            for _ in range(2000):
                if not (slot_src or where):
                    break
                for sess, is_b in ((a, False), (b, True)):
                    fin, _ = sess.step(3)
                    for sl in fin:
                        s = where.pop((is_b, sl), None)
                        if s is None:
                            s = slot_src.pop(sl)
                        out, _ = sess.read(sl, want_res=True) if k else sess.read(sl)
                        check(s, out)
    assert sorted(results) == sorted(srcs)


def test_session_ppr_round_cap_per_query(gpu_available, g15):
    """A cap of 5 rounds with epochs of 2: the epoch is cut at the cap, the query keeps
    its frontier residuals and reports the cap, as the one-launch batch does."""
    import c2g
    import oracle

    o = oracle.load_dataset(g15, "origin")
    s = int(np.argmax(np.diff(o["vlist"])))
    with c2g.Graph.load(g15, "origin") as g:
        prm = g.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0, max_iter=5)
        with c2g.Session(g, c2g.REQ_PPR, 32, prm) as sess:
            sl = sess.admit(s)
            fin = []
            for _ in range(10):
                if fin:
                    break
                fin, _ = sess.step(2)
            (pr, res), st = sess.read(sl, want_res=True)
    assert st.status_flags & c2g.FLAG_ITER_CAP and st.iterations == 5
    rp, rr, rounds, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], s, 0.15, 1e-7, max_iter=5)
    assert rounds == 5
    assert float(np.abs(pr.astype(np.float64) - rp).sum()) <= L1_TOL
    assert float(np.abs(res.astype(np.float64) - rr).sum()) <= L1_TOL


def test_session_errors(gpu_available, g15):
    import c2g

    with c2g.Graph.load(g15, "origin") as g, c2g.Session(g, c2g.REQ_SSSP, 2) as sess:
        a = sess.admit(0)
        sess.admit(1)
        with pytest.raises(c2g.C2GError) as e:
            sess.admit(2)
        assert e.value.code == c2g.ERR_OVERFLOW
        with pytest.raises(c2g.C2GError):
            sess.evict(a)  # joins at the next step: nothing to snapshot yet
        with pytest.raises(c2g.C2GError):
            sess.read(a)  # still running
        with pytest.raises(c2g.C2GError):
            sess.admit(g.V)


def test_session_snapshot_needs_the_same_push(gpu_available, g15):
    """A PPR snapshot resumes only in a session of the same push (alpha, rmax) and kind;
    elsewhere it is refused and stays the caller's."""
    import c2g

    with c2g.Graph.load(g15, "origin") as g:
        p1 = g.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)
        p2 = g.ppr_params(alpha=0.2, rmax=1e-7, seeded=0, pr0=0.2, r0=1.0)
        s = int(np.argmax(np.diff(np.fromfile(g15 + "/origin/vlist.bin", dtype=np.int32))))
        with c2g.Session(g, c2g.REQ_PPR, 32, p1) as a, c2g.Session(g, c2g.REQ_PPR, 32, p2) as b, \
                c2g.Session(g, c2g.REQ_SSSP, 32) as c:
            sl = a.admit(s)
            a.step(1)
            snap = a.evict(sl)
            for other in (b, c):
                with pytest.raises(c2g.C2GError) as e:
                    other.resume(snap)
                assert e.value.code == c2g.ERR_ARG
            sl2 = a.resume(snap)  # its own session takes it back
            fin = []
            for _ in range(200):
                fin, _ = a.step(8)
                if fin:
                    break
            assert fin == [sl2]
