"""convert2binary (utils/convert2binary.cpp:10-137): text edge lists to the origin/ files.

The library's converter (c2g_convert_text and the drop-in convert2binary program) writes
the reference converter's bytes: against a fixture made by the reference's own program
(tests/golden/make_convert_golden.py), and against a restatement of its rules on a large
seeded file whose weights come from this machine's C library rand() with the default seed,
the generator the reference calls.  Inputs on which the reference stops with an uncaught
exception or indexes out of range are format errors here, with nothing written.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import PKG

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "convert_text.npz")


def _origin(d):
    o = os.path.join(d, "origin")
    return {n: np.fromfile(os.path.join(o, n + ".bin"), np.float32 if n == "flist" else np.int32)
            for n in ("vlist", "elist", "wlist", "flist")}


def test_convert_matches_reference_fixture(built, tmp_path):
    import c2g

    g = np.load(GOLDEN)
    path = str(tmp_path / "edges.txt")
    open(path, "wb").write(g["text"].tobytes())
    mv, V, E = c2g.convert_text(path, str(tmp_path / "out"))
    out = _origin(str(tmp_path / "out"))
    assert (V, E, mv) == (len(g["vlist"]) - 1, len(g["elist"]), len(g["vlist"]) - 2)
    for n in ("vlist", "elist", "wlist", "flist"):
        assert out[n].tobytes() == g[n].tobytes(), n


def _libc_rand(n):
    libc = ctypes.CDLL("libc.so.6")
    libc.srand(1)
    libc.rand.restype = ctypes.c_int
    return np.array([libc.rand() for _ in range(n)], np.int64)


def test_convert_large_file_against_restatement(built, tmp_path):
    """200k lines over 100k ids, parsed by every host thread: rows are the sorted distinct
    destinations without self-loops, weights the C library's rand() % 100 + 1 in row order,
    flist each weight over its row's sum in double, rounded to float."""
    import c2g

    rng = np.random.default_rng(5)
    n, vmax = 200_000, 100_000
    src = rng.integers(0, vmax, n)
    lines = []
    pairs = set()
    for s in src.tolist():
        d = rng.integers(0, vmax, int(rng.integers(1, 6))).tolist()
        if rng.random() < 0.1:
            d.append(s)
        lines.append("%d %s" % (s, ":".join(map(str, d))))
        pairs.update((s, x) for x in d if x != s)
    path = str(tmp_path / "big.txt")
    open(path, "w").write("\n".join(lines) + "\n")
    mv, V, E = c2g.convert_text(path, str(tmp_path / "out"))
    out = _origin(str(tmp_path / "out"))
    e = np.array(sorted(pairs), np.int64)
    V_ref = max(max(src.tolist()), max(x for _, x in pairs)) + 1
    assert (V, E, mv) == (V_ref, len(e), V_ref - 1)
    vl = np.searchsorted(e[:, 0], np.arange(V_ref + 1))
    assert np.array_equal(out["vlist"], vl.astype(np.int32))
    assert np.array_equal(out["elist"], e[:, 1].astype(np.int32))
    w = _libc_rand(E) % 100 + 1
    assert np.array_equal(out["wlist"], w.astype(np.int32))
    row = np.repeat(np.arange(V_ref), np.diff(vl))
    sums = np.bincount(row, weights=w, minlength=V_ref)
    assert np.array_equal(out["flist"], (w / sums[row]).astype(np.float32))


@pytest.mark.parametrize("text", ["1 :2\n", "1 2::3\n", "1 x\n", "0 1\n2 3:abc\n", "-1 2\n", "1 -2\n",
                                  "1 99999999999\n", "3 4\n12:5 6\n"])
def test_convert_inputs_the_reference_cannot_take(built, tmp_path, text):
    """An empty, non-numeric or out-of-range destination (stoi throws in the reference) and a
    negative id (the reference indexes its rows with it) are format errors; nothing is
    written."""
    import c2g

    path = str(tmp_path / "bad.txt")
    open(path, "w").write(text)
    with pytest.raises(c2g.C2GError) as e:
        c2g.convert_text(path, str(tmp_path / "out"))
    assert e.value.code == c2g.ERR_FORMAT
    assert not os.path.exists(str(tmp_path / "out"))


def test_convert_lines_the_reference_skips(built, tmp_path):
    """A line without a destination token, with an id that does not fit an int, or blank is
    skipped; an empty file is one vertex and no edges."""
    import c2g

    path = str(tmp_path / "skip.txt")
    open(path, "w").write("\n7\n99999999999 3\n  \n2 1\n")
    mv, V, E = c2g.convert_text(path, str(tmp_path / "a"))
    assert (mv, V, E) == (2, 3, 1)
    open(path, "w").write("")
    assert c2g.convert_text(path, str(tmp_path / "b")) == (0, 1, 0)
    assert _origin(str(tmp_path / "b"))["vlist"].tolist() == [0, 0]


def test_convert2binary_program(built, tmp_path):
    """The drop-in program prints the reference's lines; an unreadable input prints the
    reference's message and exits 0."""
    g = np.load(GOLDEN)
    path = str(tmp_path / "edges.txt")
    open(path, "wb").write(g["text"].tobytes())
    prog = os.path.join(PKG, "bin", "convert2binary")
    r = subprocess.run([prog, path, str(tmp_path / "out")], stdout=subprocess.PIPE, stderr=subprocess.PIPE, text=True)
    assert r.returncode == 0
    V = len(g["vlist"]) - 1
    assert r.stdout.splitlines() == ["Reading graph from " + path, "Max Vertex Number: %d" % (V - 1),
                                     "Vertex Number: %d" % V, "Edge Number: %d" % len(g["elist"])]
    assert _origin(str(tmp_path / "out"))["flist"].tobytes() == g["flist"].tobytes()
    missing = str(tmp_path / "none.txt")
    r = subprocess.run([prog, missing, str(tmp_path / "o2")], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                       text=True)
    assert r.returncode == 0 and "Error opening file: " + missing in r.stderr
