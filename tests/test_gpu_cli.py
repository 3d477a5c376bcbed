"""The drop-in programs print the reference programs' lines (shape and labels, UTF-8
as the reference sources spell them) and the right results.

Line sequences follow src/sssp/base/Main.cu:22-100, src/sssp/purn/Main.cu:24-123,
src/ppr/base/Main.cu:38-110,408, src/ppr/purn/Main.cu:33-136,448 and
src/adsorption/w-base/Main.cu:39-113, with the Graph constructor / destructor lines of
src/sssp/purn/Graph.h:44-46,61.  Numbers are matched by pattern; the values are checked
against the oracle.
"""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import PKG, load_golden, write_dataset

pytestmark = pytest.mark.gpu

NUM = r"-?[0-9.e+-]+|-?nan|-?inf"
FLAG = "flag 已设置成 -1  终止条件以满足\t\titeration_num：\\d+"
SSSP_START = "==================== SSSP with FORWARD PUSH starts ============"
SSSP_END = "==================== SSSP with FORWARD PUSH ends ============"
PPR_START = "==================== PPR with FORWARD PUSH starts ===================="
PPR_END = "==================== PPR with FORWARD PUSH ends ===================="
GRAPH = ["INIT--class Graph is constructed", "The vertex num is:\\d+", "The edge num is:\\d+"]


def _run(prog, d, source):
    r = subprocess.run([os.path.join(PKG, "bin", prog), d, str(source)], stdout=subprocess.PIPE,
                       stderr=subprocess.PIPE, check=True)
    return r.stdout.decode("utf-8").split("\n")


def _shape(lines, patterns):
    """Match the output line by line against the patterns (regexes); None in the list
    matches one result line that the caller checks."""
    assert len(lines) == len(patterns) + 1 and lines[-1] == "", (len(lines), len(patterns), lines)
    for got, pat in zip(lines, patterns):
        assert re.fullmatch(pat, got), (pat, got)


@pytest.fixture(scope="module")
def gd(tmp_path_factory, built):
    g = load_golden("rmat_s12_ef8_seed5")
    return write_dataset(str(tmp_path_factory.mktemp("cli")), g), g


def test_cli_sssp_lines(gpu_available, gd):
    d, g = gd
    s = int(g["sources"][0])
    for prog, pruned in (("sssp-base", False), ("sssp-purn", True)):
        lines = _run(prog, d, s)
        res = ["\\d+\t-?\\d+"] * 10
        pat = [re.escape(d)] + GRAPH + ["Using GPU device 0", "test for study how to use cuda", "", SSSP_START]
        pat += ["", SSSP_END] if not pruned else []
        pat += [FLAG] + res + ["gpu runtime: (%s) seconds" % NUM, "源顶点source = %d" % s,
                               "CLEAR--class Graph is destroyed"]
        _shape(lines, pat)
        vals = [int(l.split("\t")[1]) for l in lines if re.fullmatch("\\d+\t-?\\d+", l)]
        want = g["dist_compat"][0] if pruned else g["dist_origin"][0]
        assert vals == want[:10].tolist(), prog


def test_cli_ppr_lines(gpu_available, gd):
    import oracle

    d, g = gd
    s = int(g["sources"][0])
    res = ["\\d+\\.\tpagerank\t (%s)\tresidual\t(%s)" % (NUM, NUM)] * 11
    for prog, pruned, ads in (("ppr-base", False, False), ("ppr-purn", True, False),
                              ("adsorption-base", False, True)):
        lines = _run(prog, d, s)
        pat = ([re.escape(d)] if pruned else []) + GRAPH + ["test for study how to use cuda", "", PPR_START]
        if pruned:
            hv, vl = g["ppr_hvlist"], g["ppr_vlist"]
            pat += ["csr_v %d--%d" % (hv[s + 1] - hv[s], vl[s + 1] - vl[s])] * 10
        pat += ["source = %dend ------------10" % s, "gpu runtime: (%s) seconds" % NUM, FLAG, PPR_END, ""]
        pat += res + ["CLEAR--class Graph is destroyed"]
        _shape(lines, pat)
        pr = np.array([float(l.split("\t")[2]) for l in lines if "\tpagerank\t" in l])
        if prog == "ppr-base":
            V = len(g["origin_vlist"]) - 1
            rp, _, _, _ = oracle.ppr_push(g["origin_vlist"], g["origin_elist"], g["origin_flist"], s, 0.2,
                                          0.001 / (V + 1), r0=1.0, pr0=0.2)
            assert np.allclose(pr, rp[:11], rtol=1e-5, atol=1e-9)
