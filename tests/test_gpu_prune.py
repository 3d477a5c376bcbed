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
    reads, and a graph without edges."""
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
