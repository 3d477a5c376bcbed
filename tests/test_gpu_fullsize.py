"""Parity at the benchmark's full size (R-MAT scale 22, edge factor 16: 4,194,304
vertices, ~65M edges, int32 weights in [1,1000], out-normalised float weights), on the
unpruned graph and on the benchmark step's own pruned inputs and sources.

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


# ---- the benchmark step itself ------------------------------------------------------
# bench.py's step: R-MAT scale 22 (seed 2) pruned by purn-sssp and by purn-ppr for alpha
# 0.15; 256 SSSP sources on sssp/ with EXACT record seeds; 256 seeded PPR sources on ppr/
# (alpha 0.15, rmax 1e-7, cap 500) at the pull ratio the autotuner picks.  The workload
# helpers are bench.py's own, so these tests check exactly what the bench times.


@pytest.fixture(scope="module")
def s22_step(tmp_path_factory, built):
    import bench
    import c2g

    d = str(tmp_path_factory.mktemp("s22step"))
    bench.make_dataset(c2g, d, 22, 16, 2)
    return d


def _pool():
    import os
    from concurrent.futures import ThreadPoolExecutor

    return ThreadPoolExecutor(max(1, min(32, os.cpu_count() or 1)))


def test_bench_step_sssp_batch_certified(gpu_available, s22_step):
    """All 256 batched rows pass the optimality certificate with their own source and
    record seeds (bit-exact shortest distances), and four rows equal the reference CPU
    Bellman-Ford restatement run from the same first hop."""
    import os

    import bench
    import c2g
    import oracle

    ds = oracle.load_dataset(s22_step, "sssp")
    src = bench.workload_sources(ds["vlist"], 256, 2024)
    with c2g.Graph.load(s22_step, "sssp") as g:
        dist, st = g.sssp_batch(src, seeds=True, mode=c2g.SEEDS_EXACT)
    assert st.status_flags == 0
    off, sv, sw = oracle.query_seeds(ds, src, "sssp")
    assert off[-1] > 0  # the step's sources carry record seeds

    def cert(i):
        return oracle.sssp_certificate(ds["vlist"], ds["elist"], ds["wlist"], dist[i], [int(src[i])],
                                       sv[off[i]:off[i + 1]], sw[off[i]:off[i + 1]])

    with _pool() as ex:
        res = list(ex.map(cert, range(len(src))))
    bad = [(i, r) for i, r in enumerate(res) if r != (0, -1)]
    assert not bad, bad[:8]
    rows = np.array([0, 77, 128, 255])
    seeds = oracle.query_seeds(ds, src[rows], "sssp")
    _, ref = oracle.batch("sssp", ds["vlist"], ds["elist"], ds["wlist"], None, src[rows],
                          threads=min(4, os.cpu_count() or 1), keep=True, seeds=seeds)
    for k, i in enumerate(rows):
        assert np.array_equal(dist[i], ref[k]), i


def test_bench_step_ppr_batch_vs_fp64(gpu_available, s22_step):
    """16 rows of the batched push (8 from the uniform half, 8 from the top-1% half) at
    the autotuned pull ratio, at ratio 16 and push-only, each within L1 1e-6 of the FP64
    oracle push (same seeds, same BSP rounds) on pr and on res."""
    import os

    import torch

    import bench
    import c2g
    import oracle

    ds = oracle.load_dataset(s22_step, "ppr")
    src = bench.workload_sources(ds["vlist"], 256, 2025)
    rows = np.concatenate([np.arange(0, 128, 16), np.arange(128, 256, 16)])
    seeds = oracle.query_seeds(ds, src[rows], "ppr")
    _, (p64, r64) = oracle.batch("ppr", ds["vlist"], ds["elist"], None, ds["wlist"], src[rows], alpha=bench.ALPHA,
                                 rmax=bench.RMAX, max_iter=500, threads=min(16, os.cpu_count() or 1), keep=True,
                                 seeds=seeds, f64=True)
    dev = torch.device("cuda", 0)
    with c2g.Graph.load(s22_step, "ppr") as g:
        prm = bench.step_ppr_params(g)
        ratio = g.ppr_batch_autotune(src, prm, reps=1)
        pr = torch.empty((len(src), g.V), dtype=torch.float32, device=dev)
        res = torch.empty((len(src), g.V), dtype=torch.float32, device=dev)
        for r in sorted({ratio, 16.0, -1.0}):
            g.ppr_batch_pull(r)
            _, _, st = g.ppr_batch(src, prm, pr_ptr=pr.data_ptr(), res_ptr=res.data_ptr())
            assert st.status_flags == 0, r
            prh = pr[torch.from_numpy(rows).to(dev)].cpu().numpy().astype(np.float64)
            resh = res[torch.from_numpy(rows).to(dev)].cpu().numpy().astype(np.float64)
            for k, i in enumerate(rows):
                lp = float(np.abs(prh[k] - p64[k]).sum())
                lr = float(np.abs(resh[k] - r64[k]).sum())
                assert lp <= L1_TOL and lr <= L1_TOL, (r, int(i), int(src[i]), lp, lr)
