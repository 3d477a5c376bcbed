"""R-MAT generation on the GPU writes the same origin/ files as the host generator,
byte for byte (endpoint draws, dedup, weights and the normalised flist)."""
import filecmp
import os

import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("scale,ef,seed,wmax", [(12, 8, 3, 100), (16, 16, 1, 100), (18, 16, 2, 1000)])
def test_rmat_gpu_matches_host(gpu_available, built, tmp_path, scale, ef, seed, wmax):
    import c2g

    host, dev = str(tmp_path / "host"), str(tmp_path / "dev")
    c2g.rmat_write(host, scale, ef, seed, 1, wmax)
    c2g.rmat_write(dev, scale, ef, seed, 1, wmax, gpu=True)
    for f in ("vlist", "elist", "wlist", "flist"):
        a, b = os.path.join(host, "origin", f + ".bin"), os.path.join(dev, "origin", f + ".bin")
        assert filecmp.cmp(a, b, shallow=False), (scale, f)


def test_streamed_load_equals_host_arrays(gpu_available, built, tmp_path):
    """c2g_graph_load streams the edge files (memory-mapped, page-locked double buffer,
    interleaved on the device in chunks of 4M edges).  At scale 19 (8.0M edges, two
    chunks, the last one partial) a loaded graph gives the same SSSP distances and PPR
    vectors as one built from the host arrays, for every variant."""
    import numpy as np

    import c2g
    import oracle

    d = str(tmp_path)
    c2g.rmat_write(d, 19, 16, 7, 1, 1000)
    c2g.prune_sssp(d)
    c2g.prune_ppr(d, alpha=0.15)
    o = oracle.load_dataset(d, "origin")
    assert (1 << 22) < len(o["elist"]) < 2 * (1 << 22)
    deg = np.diff(o["vlist"])
    srcs = [int(np.argmax(deg)), int(np.flatnonzero(deg > 0)[11])]
    with c2g.Graph.load(d, "origin") as gl, \
            c2g.Graph.create(o["vlist"], o["elist"], o["wlist"], o["flist"]) as gc:
        assert (gl.V, gl.E) == (gc.V, gc.E)
        for s in srcs:
            assert np.array_equal(gl.sssp(s)[0], gc.sssp(s)[0])
            a = gl.ppr(s, alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)[0].astype(np.float64)
            b = gc.ppr(s, alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)[0].astype(np.float64)
            assert float(np.abs(a - b).sum()) <= 1e-6  # the same push up to summation order
        ref = oracle.dijkstra(o["vlist"], o["elist"], o["wlist"], [srcs[0]], [0])
        assert np.array_equal(gl.sssp(srcs[0])[0], ref)
        pr, _, _ = gl.ppr(srcs[1], alpha=0.15, rmax=1e-7, seeded=0, pr0=0.15, r0=1.0)
        rp, _, _, _ = oracle.ppr_push(o["vlist"], o["elist"], o["flist"], srcs[1], 0.15, 1e-7)
        assert float(np.abs(pr.astype(np.float64) - rp).sum()) <= 1e-6
    for variant in ("sssp", "ppr"):
        ds = oracle.load_dataset(d, variant)
        with c2g.Graph.load(d, variant) as gl:
            assert gl.E == len(ds["elist"])
            if variant == "sssp":
                s = int(ds["hvmap"][0])
                dist, _ = gl.sssp(s, seeds=True, mode=c2g.SEEDS_EXACT)
                sv, sw = ds["helist"][ds["hvlist"][0]:ds["hvlist"][1]], ds["hwlist"][ds["hvlist"][0]:ds["hvlist"][1]]
                ref, _ = oracle.sssp_seeded(ds["vlist"], ds["elist"], ds["wlist"], s, sv, sw)
                assert np.array_equal(dist, ref)
            else:
                s = srcs[0]
                prm = gl.ppr_params(alpha=0.15, rmax=1e-7, seeded=1)
                pr, _, _ = gl.ppr(s, prm)
                seeds = oracle.query_seeds(ds, [s], "ppr")
                rp, _, _, _ = oracle.ppr_push(ds["vlist"], ds["elist"], ds["wlist"], s, 0.15, 1e-7, seeded=True,
                                              seed_v=seeds[1], seed_w=seeds[2])
                assert float(np.abs(pr.astype(np.float64) - rp).sum()) <= 1e-6


def test_streamed_load_rejects_bad_targets(gpu_available, built, tmp_path):
    """A target outside [0, V) in elist.bin is found by the device-side check of the
    streamed load (the value is compared, never used as an index) and reported as a
    format error naming the edge."""
    import numpy as np

    import c2g

    d = str(tmp_path)
    c2g.rmat_write(d, 12, 8, 3, 1, 100)
    el = np.fromfile(os.path.join(d, "origin", "elist.bin"), dtype=np.int32)
    el[777] = 4096
    el.tofile(os.path.join(d, "origin", "elist.bin"))
    with pytest.raises(c2g.C2GError) as ei:
        c2g.Graph.load(d, "origin")
    assert ei.value.code == c2g.ERR_FORMAT and "elist[777]" in str(ei.value)
