"""Parity at the benchmark's full size (R-MAT scale 22, edge factor 16: 4,194,304
vertices, ~65M edges, int32 weights in [1,1000], out-normalised float weights).

SSSP: too large for a quick Dijkstra in the test, so every result is checked with the
oracle's optimality certificate (sources at 0, no edge improves a distance, every reached
vertex has a tight in-edge): with positive weights that pins the exact shortest
distances, bit for bit.  PPR: one query against the FP64 oracle push (alpha 0.15,
rmax 1e-7, L1 <= 1e-6 on pr and res), and the batched result against the single-query
one."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
L1_TOL = 1e-6


@pytest.fixture(scope="module")
def s22(tmp_path_factory, built):
    import c2g

    d = str(tmp_path_factory.mktemp("s22"))
    c2g.rmat_write(d, 22, 16, 2, 1, 1000)
    return d


def test_sssp_fullsize_certified_single_and_batched(gpu_available, s22):
    import c2g
    import oracle

    o = oracle.load_dataset(s22, "origin")
    deg = np.diff(o["vlist"])
    rng = np.random.default_rng(22)
    top = np.argsort(-deg, kind="stable")[:len(deg) // 100]
    src = np.concatenate([rng.choice(np.flatnonzero(deg > 0), 32, replace=False),
                          rng.choice(top, 32, replace=False)]).astype(np.int32)
    with c2g.Graph.load(s22, "origin") as g:
        for s in src[[0, 40]]:
            dist, st = g.sssp(int(s))
            assert st.status_flags == 0
            assert oracle.sssp_certificate(o["vlist"], o["elist"], o["wlist"], dist, [int(s)]) == (0, -1)
        dist_b, st = g.sssp_batch(src)
        assert st.status_flags == 0
        for i in (0, 17, 40, 63):
            assert oracle.sssp_certificate(o["vlist"], o["elist"], o["wlist"], dist_b[i], [int(src[i])]) == (0, -1)
        # the batch equals the single-query kernel on the queries checked above
        d0, _ = g.sssp(int(src[0]))
        assert np.array_equal(dist_b[0], d0)


def test_ppr_fullsize_vs_fp64_and_batch(gpu_available, s22):
    import c2g
    import oracle

    o = oracle.load_dataset(s22, "origin")
    deg = np.diff(o["vlist"])
    rng = np.random.default_rng(23)
    src = rng.choice(np.flatnonzero(deg > 0), 32, replace=False).astype(np.int32)
    with c2g.Graph.load(s22, "origin") as g:
        prm = g.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)
        pr, res, st = g.ppr(int(src[0]), prm)
        assert st.status_flags == 0
        rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(src[0]), 0.15, 1e-7)
        assert np.abs(pr.astype(np.float64) - rp).sum() <= L1_TOL
        assert np.abs(res.astype(np.float64) - rr).sum() <= L1_TOL
        prb, resb, stb = g.ppr_batch(src, prm)
        assert stb.status_flags == 0
        assert np.abs(prb[0].astype(np.float64) - rp).sum() <= L1_TOL
        assert np.abs(resb[0].astype(np.float64) - rr).sum() <= L1_TOL
        pr5, _, _ = g.ppr(int(src[5]), prm)
        assert np.abs(prb[5].astype(np.float64) - pr5).sum() <= L1_TOL
