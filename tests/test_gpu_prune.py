"""purn-ppr on the GPU (c2g_prune_ppr_device) writes the same six ppr/ files as the
sequential pass, byte for byte: the oracle's restatement (oracle/ingest.c orc_prune_ppr)
and the library's host pass (c2g_prune_ppr_alpha)."""
import filecmp
import os
import shutil

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

FILES = ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist")


def _same(a, b):
    for f in FILES:
        pa, pb = os.path.join(a, "ppr", f + ".bin"), os.path.join(b, "ppr", f + ".bin")
        assert filecmp.cmp(pa, pb, shallow=False), f


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


def _write(d, vl, el, fl):
    os.makedirs(os.path.join(d, "origin"))
    np.asarray(vl, np.int32).tofile(os.path.join(d, "origin", "vlist.bin"))
    np.asarray(el, np.int32).tofile(os.path.join(d, "origin", "elist.bin"))
    np.asarray(fl, np.float32).tofile(os.path.join(d, "origin", "flist.bin"))
    np.ones(len(el), np.int32).tofile(os.path.join(d, "origin", "wlist.bin"))


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
        _write(ref, vl, el, fl)
        shutil.copytree(ref, dev)
        oracle.prune_ppr(ref, 0.15)
        c2g.prune_ppr_device(dev, 0.15)
        _same(ref, dev)


def test_prune_ppr_device_bad_alpha(gpu_available, built, tmp_path):
    import c2g

    with pytest.raises(c2g.C2GError) as e:
        c2g.prune_ppr_device(str(tmp_path), 1.5)
    assert e.value.code == c2g.ERR_ARG
    with pytest.raises(c2g.C2GError) as e:
        c2g.prune_ppr_device(str(tmp_path), 0.15)  # no origin/ files
    assert e.value.code == c2g.ERR_IO


def test_purn_ppr_program_on_the_gpu(gpu_available, built, tmp_path):
    """The drop-in purn-ppr with C2G_PRUNE_GPU=0 writes the reference factor's files (0.8),
    the same bytes as the program's host pass."""
    import subprocess

    import oracle
    from conftest import PKG

    host, dev = str(tmp_path / "host"), str(tmp_path / "dev")
    oracle.rmat_write(host, 13, 16, 9, 1, 1000)
    shutil.copytree(host, dev)
    prog = os.path.join(PKG, "bin", "purn-ppr")
    env = dict(os.environ)
    env.pop("C2G_PRUNE_GPU", None)
    subprocess.run([prog, host], check=True, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    env["C2G_PRUNE_GPU"] = "0"
    subprocess.run([prog, dev], check=True, env=env, stdout=subprocess.PIPE, stderr=subprocess.PIPE)
    _same(host, dev)
