"""Forward push on the GPU through the C ABI against the FP64 oracle (the same BSP
push, restated from calcuatePPR and pinned bit-for-bit in FP32 to the reference's CPU
push).  Tolerance: L1(pr_gpu - pr_fp64) <= 1e-6 per result (scaled by the injected
mass r0 for the adsorption program)."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, write_dataset

pytestmark = pytest.mark.gpu

L1_TOL = 1e-6


@pytest.fixture(scope="module")
def gdirs(tmp_path_factory, built):
    out = {}
    for name in golden_cases():
        g = load_golden(name)
        out[name] = (write_dataset(str(tmp_path_factory.mktemp(name)), g), g)
    return out


@pytest.fixture(scope="module")
def rmat14(tmp_path_factory, built):
    import c2g

    d = str(tmp_path_factory.mktemp("rmat14"))
    c2g.rmat_write(d, 14, 16, 2, 1, 1000)
    c2g.prune_ppr(d)
    return d


def l1(a, b):
    return float(np.abs(a.astype(np.float64) - b).sum())


@pytest.mark.parametrize("pull_div", [0, 8, 1 << 30])
@pytest.mark.parametrize("alpha,rmax", [(0.15, 1e-7), (0.2, None), (0.15, 1e-5)])
def test_ppr_base_vs_fp64(gpu_available, gdirs, rmat14, alpha, rmax, pull_div):
    """Push-only, mixed push/pull and pull-every-round give the same BSP rounds."""
    import c2g
    import oracle

    dirs = [d for d, _ in gdirs.values()] + [rmat14]
    for d in dirs:
        o = oracle.load_dataset(d, "origin")
        V = len(o["vlist"]) - 1
        rm = rmax if rmax is not None else 0.001 / (V + 1)
        deg = np.diff(o["vlist"])
        srcs = [int(np.argmax(deg)), int(np.flatnonzero(deg > 0)[-1])]
        with c2g.Graph.load(d, "origin") as gr:
            gr.ppr_config(pull_div=pull_div)
            for s in srcs:
                p = gr.ppr_params(alpha=alpha, rmax=rm, r0=1.0, pr0=alpha, seeded=0, max_iter=500)
                pr, res, st = gr.ppr(s, p)
                rp, rr, rounds, cnt = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], s, alpha, rm)
                assert l1(pr, rp) <= L1_TOL, (d, s, l1(pr, rp))
                assert l1(res, rr) <= L1_TOL, (d, s, l1(res, rr))
                assert abs(st.iterations - rounds) <= 2
                assert st.status_flags == 0


@pytest.mark.parametrize("pull_div", [0, 8])
def test_ppr_seeded_pruned_vs_fp64(gpu_available, gdirs, rmat14, pull_div):
    """ppr-purn: pruned ppr/ graph, first hop = the source's records + kept edges."""
    import c2g
    import oracle

    for d in [d for d, _ in gdirs.values()] + [rmat14]:
        p = oracle.load_dataset(d, "ppr")
        hv, he, hw = p["hvlist"], p["helist"], p["hwlist"]
        V = len(p["vlist"]) - 1
        deg = np.diff(p["vlist"])
        cand = [int(np.argmax(deg))] + [int(v) for v in np.flatnonzero(np.diff(hv) > 0)[:3]]
        with c2g.Graph.load(d, "ppr") as gr:
            gr.ppr_config(pull_div=pull_div)
            for s in cand:
                for alpha, rm in ((0.2, 0.001 / (V + 1)), (0.15, 1e-7)):
                    prm = gr.ppr_params(alpha=alpha, rmax=rm, seeded=1)
                    pr, res, st = gr.ppr(s, prm)
                    sv = np.concatenate([he[hv[s]:hv[s + 1]], p["elist"][p["vlist"][s]:p["vlist"][s + 1]]])
                    sw = np.concatenate([hw[hv[s]:hv[s + 1]], p["wlist"][p["vlist"][s]:p["vlist"][s + 1]]])
                    rp, rr, _, _ = oracle.ppr_push(p["vlist"], p["elist"], p["wlist"], s, alpha, rm, seeded=True,
                                                   seed_v=sv, seed_w=sw)
                    assert l1(pr, rp) <= L1_TOL, (d, s, alpha, l1(pr, rp))
                    assert l1(res, rr) <= L1_TOL
                    assert st.n_seeds == len(sv)


def test_adsorption_program_vs_fp64(gpu_available, rmat14):
    """The reference adsorption program: residual 10, pr += 0.8*10, rmax = 1/V, cap 2000."""
    import c2g
    import oracle

    o = oracle.load_dataset(rmat14, "origin")
    V = len(o["vlist"]) - 1
    s = int(np.argmax(np.diff(o["vlist"])))
    with c2g.Graph.load(rmat14, "origin") as gr:
        prm = gr.ppr_params(adsorption=True)
        assert abs(prm.r0 - 10) < 1e-6 and abs(prm.pr0 - 8) < 1e-6 and prm.max_iter == 2000
        pr, res, _ = gr.ppr(s, prm)
        rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], s, 0.2, float(np.float32(1.0 / V)),
                                       r0=10.0, pr0=8.0, max_iter=2000)
        assert l1(pr, rp) <= L1_TOL * 10
        assert l1(res, rr) <= L1_TOL * 10


def test_ppr_round_cap_keeps_residual(gpu_available, rmat14):
    import c2g
    import oracle

    o = oracle.load_dataset(rmat14, "origin")
    s = int(np.argmax(np.diff(o["vlist"])))
    with c2g.Graph.load(rmat14, "origin") as gr:
        for cap in (1, 3):
            prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, max_iter=cap)
            pr, res, st = gr.ppr(s, prm)
            assert st.status_flags & c2g.FLAG_ITER_CAP
            rp, rr, rounds, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], s, 0.15, 1e-7, max_iter=cap)
            assert rounds == cap
            assert l1(pr, rp) <= L1_TOL and l1(res, rr) <= L1_TOL


def test_ppr_device_output_and_repeat(gpu_available, rmat14):
    import torch

    import c2g
    import oracle

    o = oracle.load_dataset(rmat14, "origin")
    deg = np.diff(o["vlist"])
    srcs = np.flatnonzero(deg > 0)[:: max(1, len(deg) // 12)][:12]
    with c2g.Graph.load(rmat14, "origin") as gr:
        prm = gr.ppr_params(alpha=0.15, rmax=1e-6, seeded=0, pr0=0.15)
        pr_d = torch.empty(gr.V, dtype=torch.float32, device="cuda:0")
        for s in srcs:
            gr.ppr(int(s), prm, pr_ptr=pr_d.data_ptr())
            rp, _, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(s), 0.15, 1e-6)
            assert l1(pr_d.cpu().numpy(), rp) <= L1_TOL, s


def test_ppr_dangling_source(gpu_available):
    import c2g

    vl = np.array([0, 2, 2, 3], np.int32)
    el = np.array([1, 2, 0], np.int32)
    fl = np.array([0.5, 0.5, 1.0], np.float32)
    with c2g.Graph.create(vl, el, flist=fl) as gr:
        prm = gr.ppr_params(alpha=0.2, rmax=1e-9, seeded=0, pr0=0.2)
        pr, res, st = gr.ppr(1, prm)       # no out-edges: only the source's own share
        assert np.allclose(pr, [0, 0.2, 0]) and np.allclose(res, 0)
        pr, res, st = gr.ppr(0, prm)
        assert pr[0] > 0.2 and pr.sum() <= 1.0 + 1e-6


def test_ppr_many_sources_fp64_parity(gpu_available, rmat14):
    """Forty sources on one handle: every result within L1 1e-6 of the FP64 oracle in pr
    and res (FP64 residual bookkeeping keeps threshold decisions with the oracle)."""
    import c2g
    import oracle

    o = oracle.load_dataset(rmat14, "origin")
    deg = np.diff(o["vlist"])
    rng = np.random.default_rng(21)
    srcs = rng.choice(np.flatnonzero(deg > 0), 40, replace=False)
    with c2g.Graph.load(rmat14, "origin") as gr:
        prm = gr.ppr_params(alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)
        for s in srcs:
            pr, res, _ = gr.ppr(int(s), prm)
            rp, rr, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], int(s), 0.15, 1e-7)
            assert l1(pr, rp) <= L1_TOL and l1(res, rr) <= L1_TOL, (s, l1(pr, rp), l1(res, rr))
