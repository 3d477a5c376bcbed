"""The C-ABI library: it loads, exports every symbol include/c2graph.h declares, and
fails with status codes (never exit) on host-side errors.  No GPU compute here."""
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import PKG, REPO


def declared_symbols():
    text = open(os.path.join(REPO, "include", "c2graph.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(c2g_[a-z0-9_]+)\s*\(", text)))


def test_header_symbols_exported(built):
    import c2g

    L = c2g.lib()
    names = declared_symbols()
    assert len(names) >= 17
    for n in names:
        assert hasattr(L, n), n
        assert n in c2g.SIGNATURES, "binding lacks " + n
    out = subprocess.run(["nm", "-D", "--defined-only", c2g.LIB_PATH], stdout=subprocess.PIPE,
                         text=True, check=True).stdout
    exported = set(re.findall(r" T (c2g_\w+)", out))
    assert set(names) <= exported


def test_abi_version(built):
    import c2g

    assert c2g.lib().c2g_abi_version() == 2


def test_missing_dataset_is_io_error(built, tmp_path):
    import c2g

    with pytest.raises(c2g.C2GError) as e:
        c2g.Graph.load(str(tmp_path / "nope"), "sssp")
    assert e.value.code == c2g.ERR_IO
    assert "not exist" in str(e.value)


def test_bad_variant_and_args(built, tmp_path):
    import ctypes

    import c2g

    h = ctypes.c_void_p()
    assert c2g.lib().c2g_graph_load(b"/x", 7, 0, ctypes.byref(h)) == c2g.ERR_ARG
    assert c2g.lib().c2g_graph_load(None, 0, 0, ctypes.byref(h)) == c2g.ERR_ARG
    assert c2g.lib().c2g_sssp(None, 0, 0, 0, None, 0, None) == c2g.ERR_ARG
    assert c2g.lib().c2g_prune_sssp(None) == c2g.ERR_ARG
    assert c2g.lib().c2g_prune_ppr_device(None, 0.15, 0, None, None, None) == c2g.ERR_ARG
    assert c2g.lib().c2g_prune_sssp_device(None, 0, None, None, None) == c2g.ERR_ARG
    assert c2g.lib().c2g_convert_text(None, b"/tmp/x", None, None, None) == c2g.ERR_ARG
    assert c2g.lib().c2g_rmat_write(b"/tmp/x", 0, 8, 1, 1, 10, 0.57, 0.19, 0.19) == c2g.ERR_ARG
    # batched-query tuning entry points: a NULL handle or batch is a status, never a crash
    assert c2g.lib().c2g_ppr_batch_set_pull(None, 8.0) == c2g.ERR_ARG
    assert c2g.lib().c2g_sssp_batch_set_pull(None, 0.5) == c2g.ERR_ARG
    src = np.zeros(4, dtype=np.int32)
    prm = c2g.PprParams()
    assert c2g.lib().c2g_ppr_batch_autotune(None, 4, c2g._ptr(src), ctypes.byref(prm), 1, None, None) == c2g.ERR_ARG
    assert c2g.lib().c2g_sssp_autotune(None, 4, c2g._ptr(src), 0, 0, None, None, None) == c2g.ERR_ARG
    assert c2g.lib().c2g_rmat_write_gpu(None, 10, 8, 1, 1, 10, 0.57, 0.19, 0.19, 0) == c2g.ERR_ARG


def test_corrupt_dataset_is_format_error(built, tmp_path):
    """A truncated or non-monotone CSR is rejected before any device work."""
    import c2g

    d = tmp_path / "bad"
    (d / "origin").mkdir(parents=True)
    np.array([0, 3, 2, 4], dtype=np.int32).tofile(str(d / "origin" / "vlist.bin"))
    np.array([1, 2, 0, 1], dtype=np.int32).tofile(str(d / "origin" / "elist.bin"))
    np.array([1, 1, 1, 1], dtype=np.int32).tofile(str(d / "origin" / "wlist.bin"))
    with pytest.raises(c2g.C2GError) as e:
        c2g.Graph.load(str(d), "origin")
    assert e.value.code == c2g.ERR_FORMAT
    open(str(d / "origin" / "elist.bin"), "wb").write(b"\x01\x00\x00")  # not a multiple of 4
    with pytest.raises(c2g.C2GError) as e:
        c2g.Graph.load(str(d), "origin")
    assert e.value.code == c2g.ERR_FORMAT


def test_prune_missing_input(built, tmp_path):
    import c2g

    with pytest.raises(c2g.C2GError) as e:
        c2g.prune_sssp(str(tmp_path))
    assert e.value.code == c2g.ERR_IO


def test_cli_missing_file_exits_zero(built, tmp_path):
    """Reference behaviour (core/io.hpp:27-30): message on stderr, exit 0."""
    for prog in ("sssp-base", "sssp-purn", "ppr-purn"):
        r = subprocess.run([os.path.join(PKG, "bin", prog), str(tmp_path), "0"], stdout=subprocess.PIPE,
                           stderr=subprocess.PIPE, text=True)
        assert r.returncode == 0, prog
        assert "not exist" in r.stderr, prog


def test_cli_prune_matches_library(built, tmp_path):
    import c2g

    for sub in ("a", "b"):
        c2g.rmat_write(str(tmp_path / sub), 9, 8, 4, 1, 100)
    subprocess.run([os.path.join(PKG, "bin", "purn-sssp"), str(tmp_path / "a")], check=True,
                   stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    c2g.prune_sssp(str(tmp_path / "b"))
    for n in ("vlist", "elist", "wlist", "hvlist", "helist", "hwlist", "hvmap"):
        assert (tmp_path / "a" / "sssp" / (n + ".bin")).read_bytes() == \
               (tmp_path / "b" / "sssp" / (n + ".bin")).read_bytes()


def test_no_device_is_reported(built):
    """Without a GPU the library reports NODEVICE instead of falling back."""
    import c2g

    if c2g.device_count() > 0:
        pytest.skip("a GPU is present")
    g = __import__("conftest").load_golden("tiny12")
    with pytest.raises(c2g.C2GError) as e:
        c2g.Graph.create(g["origin_vlist"], g["origin_elist"], g["origin_wlist"])
    assert e.value.code == c2g.ERR_NODEVICE


def test_device_pruners_fail_loudly_without_a_gpu(built, tmp_path):
    """Without a usable GPU the device pruners return a CUDA error and write nothing: no
    silent fallback to a host pass."""
    import torch

    import c2g
    import oracle

    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    d = str(tmp_path)
    oracle.rmat_write(d, 10, 8, 1, 1, 100)
    for kind, fn in (("ppr", lambda: c2g.prune_ppr_device(d, 0.15)), ("sssp", lambda: c2g.prune_sssp_device(d))):
        with pytest.raises(c2g.C2GError) as e:
            fn()
        assert e.value.code == c2g.ERR_CUDA
        assert not os.path.exists(os.path.join(d, kind, "vlist.bin"))
