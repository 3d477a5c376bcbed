"""Generate tests/golden/convert_text.npz from the reference's own convert2binary
(utils/convert2binary.cpp, built into oracle/_ref/ from the reference sources).

Run where the reference tree is mounted:   python tests/golden/make_convert_golden.py

The input is a seeded text edge list in the reference's format ("src dst:dst:..." per
line) with the cases its reader handles: repeated and unsorted destinations, self-loops,
blank lines, lines without destinations, a trailing ':', a second token on a line (ignored),
signed and zero-padded ids, tabs and CR-LF line ends, and a gap of ids with no edges.  The
fixture holds the text and the four origin/ arrays the reference writes for it.
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)

from oracle import build as obuild  # noqa: E402


def make_text(seed=11, n_src=400, max_id=1500):
    rng = np.random.default_rng(seed)
    lines = []
    for _ in range(n_src):
        s = int(rng.integers(0, max_id))
        k = int(rng.integers(1, 12))
        d = rng.integers(0, max_id, k).tolist()
        if rng.random() < 0.2:
            d.append(s)  # a self-loop
        if rng.random() < 0.3:
            d.extend(d[:2])  # repeats
        lines.append("%d %s" % (s, ":".join(str(x) for x in d)))
    lines += ["", "17", "  42\t7:8:9:", "5 6:7 8:9", "+3 4", "-0 2", "9 010:0011", "12 13:14\r",
              "%d 1" % (max_id + 500), "\t\t", "1000000"]
    order = rng.permutation(len(lines))
    return "\n".join(lines[i] for i in order) + "\n"


def main():
    obuild.build_ref()
    tool = os.path.join(REPO, "oracle", "_ref", "convert2binary")
    text = make_text()
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "edges.txt")
        open(path, "w").write(text)
        os.makedirs(os.path.join(d, "out", "origin"))
        subprocess.run([tool, path, os.path.join(d, "out")], check=True, stdout=subprocess.DEVNULL)
        o = os.path.join(d, "out", "origin")
        arrays = {n: np.fromfile(os.path.join(o, n + ".bin"), np.float32 if n == "flist" else np.int32)
                  for n in ("vlist", "elist", "wlist", "flist")}
    np.savez_compressed(os.path.join(HERE, "convert_text.npz"), text=np.frombuffer(text.encode(), np.uint8),
                        **arrays)
    print("wrote convert_text.npz: V=%d E=%d" % (len(arrays["vlist"]) - 1, len(arrays["elist"])))


if __name__ == "__main__":
    main()
