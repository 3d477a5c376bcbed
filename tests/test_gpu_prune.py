"""purn-ppr and purn-sssp on the GPU (c2g_prune_ppr_device, c2g_prune_sssp_device) write the
same files as the sequential passes, byte for byte: the oracle's restatements
(oracle/ingest.c orc_prune_ppr, orc_prune_sssp) and the library's host passes
(c2g_prune_ppr_alpha, c2g_prune_sssp)."""
import filecmp
import os
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FILES = {"ppr": ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist"),
         "sssp": ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist", "hvmap")}


def _same(a, b, kind="ppr"):
    for f in FILES[kind]:
        pa, pb = os.path.join(a, kind, f + ".bin"), os.path.join(b, kind, f + ".bin")
        assert filecmp.cmp(pa, pb, shallow=False), (kind, f)


@pytest.mark.parametrize("scale,ef,seed,alpha", [(10, 8, 1, None), (14, 16, 5, 0.15), (17, 16, 2, 0.15)])
def test_prune_ppr_device_matches_sequential(gpu_available, built, tmp_path, scale, ef, seed, alpha):
    import c2g
    import oracle

    ref, host, dev = str(tmp_path / "ref"), str(tmp_path / "host"), str(tmp_path / "dev")
    oracle.rmat_write(ref, scale, ef, seed, 1, 1000)
    shutil.copytree(ref, host)
    shutil.copytree(ref, dev)
    oracle.prune_ppr(ref, alpha)
    c2g.prune_ppr(host, alpha)
    ms, rounds = c2g.prune_ppr_device(dev, 0.2 if alpha is None else alpha)
    _same(ref, dev)
    _same(host, dev)
    V = 1 << scale
    assert 0 < rounds < V // 4 and ms > 0.0


@pytest.mark.parametrize("scale,ef,seed", [(10, 8, 1), (14, 16, 5), (17, 16, 2)])
def test_prune_sssp_device_matches_sequential(gpu_available, built, tmp_path, scale, ef, seed):
    """purn-sssp's visits in rounds k = 1..29; the records in visiting order with the
    record->vertex sidecar."""
    import c2g
    import oracle

    ref, host, dev = str(tmp_path / "ref"), str(tmp_path / "host"), str(tmp_path / "dev")
    oracle.rmat_write(ref, scale, ef, seed, 1, 1000)
    shutil.copytree(ref, host)
    shutil.copytree(ref, dev)
    oracle.prune_sssp(ref)
    c2g.prune_sssp(host)
    ms, rounds = c2g.prune_sssp_device(dev)
    _same(ref, dev, "sssp")
    _same(host, dev, "sssp")
    assert rounds > 0 and ms > 0.0


def _write(d, vl, el, fl, wl=None):
    os.makedirs(os.path.join(d, "origin"))
    np.asarray(vl, np.int32).tofile(os.path.join(d, "origin", "vlist.bin"))
    np.asarray(el, np.int32).tofile(os.path.join(d, "origin", "elist.bin"))
    np.asarray(fl, np.float32).tofile(os.path.join(d, "origin", "flist.bin"))
    (np.ones(len(el), np.int32) if wl is None else np.asarray(wl, np.int32)).tofile(
        os.path.join(d, "origin", "wlist.bin"))


def test_prune_ppr_device_edge_cases(gpu_available, built, tmp_path):
    """Repeated targets with different weights (kept as separate pairs, merged one by
    one), self-loops (dropped), a chain whose visits each rewrite the row the next one
    reads, a graph without edges, and unsorted rows with repeated pairs."""
    import c2g
    import oracle

    rng = np.random.default_rng(3)
    cases = {}
    # duplicates and self-loops on a small random graph
    V = 64
    src = rng.integers(0, V, 600)
    dst = np.where(rng.random(600) < 0.3, (src + 1) % V, rng.integers(0, V, 600))
    dst[::37] = src[::37]
    o = np.lexsort((dst, src))
    src, dst = src[o], dst[o]
    f = rng.choice(np.array([0.25, 0.5, 0.125], np.float32), 600)
    cases["dup"] = (np.searchsorted(src, np.arange(V + 1)), dst, f)
    # a chain 0 -> 1 -> ... -> 39
    n = 40
    cases["chain"] = (np.concatenate([np.arange(n), [n - 1]]), np.arange(1, n),
                      np.linspace(0.1, 0.9, n - 1).astype(np.float32))
    cases["empty"] = (np.zeros(9, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32))
    # an R-MAT graph with every row shuffled and some pairs repeated: the rows are sorted and
    # deduplicated before the visits (the R-MAT writer's own rows are taken as they are)
    g = str(tmp_path / "rmat")
    oracle.rmat_write(g, 12, 16, 4, 1, 1000)
    o = oracle.load_dataset(g, "origin")
    vl, el, fl = o["vlist"], o["elist"].copy(), o["flist"].copy()
    rows_e, rows_f = [], []
    for v in range(len(vl) - 1):
        e, f = el[vl[v]:vl[v + 1]], fl[vl[v]:vl[v + 1]]
        if len(e) > 2 and v % 3 == 0:
            e, f = np.concatenate([e, e[:2]]), np.concatenate([f, f[:2]])
        q = rng.permutation(len(e))
        rows_e.append(e[q])
        rows_f.append(f[q])
    cases["shuffled"] = (np.concatenate([[0], np.cumsum([len(e) for e in rows_e])]), np.concatenate(rows_e),
                         np.concatenate(rows_f))
    for name, (vl, el, fl) in cases.items():
        ref, dev = str(tmp_path / (name + "_ref")), str(tmp_path / (name + "_dev"))
        # int weights with repeats, so that purn-sssp's rows also hold repeated targets
        _write(ref, vl, el, fl, rng.integers(1, 6, len(el)))
        shutil.copytree(ref, dev)
        oracle.prune_ppr(ref, 0.15)
        c2g.prune_ppr_device(dev, 0.15)
        _same(ref, dev, "ppr")
        try:
            oracle.prune_sssp(ref)
        except RuntimeError:  # the pass stops ("something error2"): so does the device
            with pytest.raises(c2g.C2GError) as e:
                c2g.prune_sssp_device(dev)
            assert e.value.code == c2g.ERR_FORMAT
            continue
        c2g.prune_sssp_device(dev)
        _same(ref, dev, "sssp")


def test_prune_device_stops_where_the_pass_stops(gpu_available, built, tmp_path):
    """Two pairs 1 -> 2 with different weights each kill 1's entry in 2's in-row, so 2's
    live in-degree (1) falls below its live roots (0 and 3): both pruners stop at 2's visit
    ("something error2", src/purn-sssp.cpp:151-166), the host passes and the device alike,
    and nothing is written."""
    import c2g
    import oracle

    vl, el = [0, 1, 3, 4, 5, 5], [1, 2, 2, 4, 2]
    d = str(tmp_path / "g")
    _write(d, vl, el, [0.5, 0.25, 0.75, 0.5, 0.5], [1, 1, 2, 1, 1])
    for kind in ("ppr", "sssp"):
        with pytest.raises(RuntimeError):
            oracle.prune_ppr(d, 0.15) if kind == "ppr" else oracle.prune_sssp(d)
        with pytest.raises(c2g.C2GError) as e:
            c2g.prune_ppr(d, 0.15) if kind == "ppr" else c2g.prune_sssp(d)
        assert e.value.code == c2g.ERR_FORMAT
        shutil.rmtree(os.path.join(d, kind), ignore_errors=True)
        with pytest.raises(c2g.C2GError) as e:
            c2g.prune_ppr_device(d, 0.15) if kind == "ppr" else c2g.prune_sssp_device(d)
        assert e.value.code == c2g.ERR_FORMAT
        assert not os.path.exists(os.path.join(d, kind))


def test_prune_ppr_device_bad_alpha(gpu_available, built, tmp_path):
    import c2g

    with pytest.raises(c2g.C2GError) as e:
        c2g.prune_ppr_device(str(tmp_path), 1.5)
    assert e.value.code == c2g.ERR_ARG
    with pytest.raises(c2g.C2GError) as e:
        c2g.prune_ppr_device(str(tmp_path), 0.15)  # no origin/ files
    assert e.value.code == c2g.ERR_IO


def test_prune_programs_on_the_gpu(gpu_available, built, tmp_path):
    """The drop-in purn-ppr and purn-sssp with C2G_PRUNE_GPU=0 write the same bytes as the
    programs' host passes (purn-ppr with the reference factor 0.8)."""
    import subprocess

    import oracle
    from conftest import PKG

    host, dev = str(tmp_path / "host"), str(tmp_path / "dev")
    oracle.rmat_write(host, 13, 16, 9, 1, 1000)
    shutil.copytree(host, dev)
    env = dict(os.environ)
    for name in ("purn-ppr", "purn-sssp"):
        prog = os.path.join(PKG, "bin", name)
        env.pop("C2G_PRUNE_GPU", None)
        subprocess.run([prog, host], check=True, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
        env["C2G_PRUNE_GPU"] = "0"
        subprocess.run([prog, dev], check=True, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    _same(host, dev, "ppr")
    _same(host, dev, "sssp")


def test_prune_device_on_small_random_graphs(gpu_available, built, tmp_path):
    """40 seeded random graphs of 20-300 vertices with self-loops, half of them with repeated
    targets of different weights: both device pruners write the oracle's bytes, or stop with
    a format error where the sequential pass stops, writing nothing."""
    import c2g
    import oracle

    rng = np.random.default_rng(23)
    done, stops = 0, 0
    for case in range(40):
        V = int(rng.integers(20, 300))
        m = int(rng.integers(V, 6 * V))
        src = np.sort(rng.integers(0, V, m))
        dst = np.where(rng.random(m) < 0.5, rng.integers(0, max(2, V // 10), m), rng.integers(0, V, m))
        order = np.lexsort((dst, src))
        src, dst = src[order], dst[order]
        if case % 2 == 0:
            keep = np.concatenate([[True], (src[1:] != src[:-1]) | (dst[1:] != dst[:-1])])
            src, dst = src[keep], dst[keep]
        ref, dev = str(tmp_path / ("r%d" % case)), str(tmp_path / ("d%d" % case))
        _write(ref, np.searchsorted(src, np.arange(V + 1)), dst,
               rng.choice(np.array([0.25, 0.5, 0.75], np.float32), len(dst)), rng.integers(1, 4, len(dst)))
        shutil.copytree(ref, dev)
        for kind in ("ppr", "sssp"):
            try:
                oracle.prune_ppr(ref, 0.15) if kind == "ppr" else oracle.prune_sssp(ref)
            except RuntimeError:
                with pytest.raises(c2g.C2GError) as e:
                    c2g.prune_ppr_device(dev, 0.15) if kind == "ppr" else c2g.prune_sssp_device(dev)
                assert e.value.code == c2g.ERR_FORMAT
                assert not os.path.exists(os.path.join(dev, kind, "vlist.bin"))
                stops += 1
                continue
            c2g.prune_ppr_device(dev, 0.15) if kind == "ppr" else c2g.prune_sssp_device(dev)
            _same(ref, dev, kind)
            done += 1
    assert done >= 40 and stops > 0, (done, stops)
