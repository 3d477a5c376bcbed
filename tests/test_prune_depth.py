"""Dependency depth of the pruners' visiting order (oracle/ingest.c orc_prune_depth).

The pruners visit vertices in a fixed sequential order, and a visit reads and writes
rows (out-rows of the vertex and its roots, in-rows of the targets it moves) that later
visits read.  The analysis gives every visit the level one past the latest visit it
depends on (read-after-write, write-after-read, write-after-write); the largest level is
the fewest steps in which a parallel pruner that reproduces the sequential bytes could
run.  These tests check that the analysis leaves the outputs unchanged and that its
counts are consistent; the figures at scale 22 are quoted with the command that makes
them in the design notes.
"""
import filecmp
import os

import pytest


@pytest.mark.parametrize("kind", ["sssp", "ppr"])
def test_prune_depth_outputs_and_counts(tmp_path, kind):
    import oracle

    a, b = str(tmp_path / "a"), str(tmp_path / "b")
    for d in (a, b):
        oracle.rmat_write(d, 14, 16, 5, 1, 1000)
    st = oracle.prune_depth(a, kind, 0.15 if kind == "ppr" else None)
    if kind == "ppr":
        oracle.prune_ppr(b, 0.15)
    else:
        oracle.prune_sssp(b)
    names = sorted(os.listdir(os.path.join(b, kind)))
    assert names == sorted(os.listdir(os.path.join(a, kind)))
    for f in names:  # the analysis does not change what the pruner writes
        assert filecmp.cmp(os.path.join(a, kind, f), os.path.join(b, kind, f), shallow=False), f
    assert 0 < st["removing"] <= st["visits"]
    assert st["visit_depth"] <= st["depth"]
    # a chain cannot be longer than the operations in it (visits plus decisions) ...
    assert st["depth"] <= st["visits"] + st["decisions"]
    # ... and the levels hold every visit once
    assert st["widest"] <= st["visits"] and st["in_levels_ge1024"] <= st["in_levels_ge32"] <= st["visits"]
    # the order is far from a single chain even at this scale
    assert st["visits"] >= 8 * st["visit_depth"]


def test_prune_depth_of_a_chain_is_sequential(tmp_path):
    """A path 0 -> 1 -> ... -> n-1 pruned by purn-sssp.  Vertex 1's visit moves its edge
    1 -> 2 into vertex 0's row, so vertex 2's only live root becomes 0, and so on: every
    visit reads and rewrites row 0 after the one before it.  The visits form one chain,
    which starts after vertex 0's own decision (it is not pruned) has read row 0."""
    import numpy as np

    import oracle

    d = str(tmp_path / "chain")
    n = 40
    vl = np.concatenate([np.arange(n, dtype=np.int32), [n - 1]]).astype(np.int32)
    el = np.arange(1, n, dtype=np.int32)
    wl = np.arange(1, n, dtype=np.int32)
    os.makedirs(os.path.join(d, "origin"))
    for name, arr in (("vlist", vl), ("elist", el), ("wlist", wl)):
        arr.tofile(os.path.join(d, "origin", name + ".bin"))
    st = oracle.prune_depth(d, "sssp")
    assert st["visits"] == n - 2  # vertices 1 .. n-2 have one root and an out-edge
    assert st["removing"] == st["visits"] and st["visit_depth"] == st["visits"] + 1


@pytest.mark.parametrize("alpha,window", [(None, 64), (0.15, 1024)])
def test_prune_ppr_speculative_schedule_reproduces_the_bytes(tmp_path, alpha, window):
    """purn-ppr's visits in rounds of the reservation-based schedule a parallel pruner
    would run (every vertex visited once, committed out of id order) write the same bytes
    as the sequential pass, in far fewer rounds than visits."""
    import oracle

    d = str(tmp_path / "g")
    oracle.rmat_write(d, 14, 16, 6, 1, 1000)
    oracle.prune_ppr(d, alpha)
    st = oracle.prune_ppr_speculative(d, alpha, window)
    for f in ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist"):
        assert filecmp.cmp(os.path.join(d, "ppr", f + ".bin"), os.path.join(d, "ppr_spec", f + ".bin"),
                           shallow=False), f
    V = 1 << 14
    assert st["visits"] == V
    assert st["rounds"] * 8 < V and st["widest"] > 32


@pytest.mark.parametrize("kind,window", [("sssp", 4096), ("sssp", 64), ("ppr", 3072)])
def test_prune_speculative_schedule_reproduces_the_bytes(tmp_path, kind, window):
    """Both pruners' steps in rounds of the device pruners' schedule (a window of positions
    from the first pending one; purn-sssp's positions are (round k, vertex)) write the same
    bytes as the sequential passes, the record->vertex sidecar included."""
    import oracle

    d = str(tmp_path / "g")
    oracle.rmat_write(d, 14, 16, 6, 1, 1000)
    if kind == "ppr":
        oracle.prune_ppr(d, 0.15)
    else:
        oracle.prune_sssp(d)
    st = oracle.prune_speculative(d, kind, 0.15 if kind == "ppr" else None, window)
    names = ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist") + (("hvmap",) if kind == "sssp" else ())
    for f in names:
        assert filecmp.cmp(os.path.join(d, kind, f + ".bin"), os.path.join(d, kind + "_spec", f + ".bin"),
                           shallow=False), f
    positions = (1 if kind == "ppr" else 29) << 14
    assert st["rounds"] < positions // window + 4096 and st["widest"] > 32


def test_speculative_schedule_on_small_random_graphs(tmp_path):
    """60 seeded random graphs of 20-300 vertices with self-loops, half of them with repeated
    targets of different weights, windows of 1 to V positions: the schedule writes the
    sequential pass's bytes for both pruners, or stops where the sequential pass stops
    ("something error2", which repeated targets cause)."""
    import numpy as np

    import oracle

    rng = np.random.default_rng(17)
    stops, done = 0, {"ppr": 0, "sssp": 0}
    for case in range(60):
        V = int(rng.integers(20, 300))
        m = int(rng.integers(V, 6 * V))
        src = np.sort(rng.integers(0, V, m))
        hub = rng.integers(0, max(2, V // 10), m)
        dst = np.where(rng.random(m) < 0.5, hub, rng.integers(0, V, m))
        order = np.lexsort((dst, src))
        src, dst = src[order], dst[order]
        if case % 2 == 0:  # distinct targets per row: no pair repeats a target
            keep = np.concatenate([[True], (src[1:] != src[:-1]) | (dst[1:] != dst[:-1])])
            src, dst = src[keep], dst[keep]
            m = len(src)
        d = str(tmp_path / ("g%d" % case))
        os.makedirs(os.path.join(d, "origin"))
        np.searchsorted(src, np.arange(V + 1)).astype(np.int32).tofile(os.path.join(d, "origin", "vlist.bin"))
        dst.astype(np.int32).tofile(os.path.join(d, "origin", "elist.bin"))
        rng.integers(1, 4, m).astype(np.int32).tofile(os.path.join(d, "origin", "wlist.bin"))
        rng.choice(np.array([0.25, 0.5, 0.75], np.float32), m).tofile(os.path.join(d, "origin", "flist.bin"))
        window = int(rng.choice([1, 3, 16, 64, V]))  # V: every position of the graph in one window
        for kind in ("ppr", "sssp"):
            try:
                oracle.prune_ppr(d, 0.15) if kind == "ppr" else oracle.prune_sssp(d)
            except RuntimeError:
                with pytest.raises(RuntimeError):
                    oracle.prune_speculative(d, kind, 0.15 if kind == "ppr" else None, window)
                stops += 1
                continue
            oracle.prune_speculative(d, kind, 0.15 if kind == "ppr" else None, window)
            names = ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist") + (("hvmap",) if kind == "sssp" else ())
            for f in names:
                assert filecmp.cmp(os.path.join(d, kind, f + ".bin"), os.path.join(d, kind + "_spec", f + ".bin"),
                                   shallow=False), (case, kind, f)
            done[kind] += 1
    assert done["ppr"] >= 20 and done["sssp"] >= 20 and stops > 0, (done, stops)
