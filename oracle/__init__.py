"""CPU oracle for the C^2graph traversal path -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import this
package, as the checker or as the timed CPU baseline; the product library
(c-2graph_gb300) never does.  The functions wrap oracle/oracle.c (a plain-C
restatement of the reference algorithms, each citing the reference file:line it
follows) and read the reference's binary dataset layout with numpy.
"""
import ctypes
import os

import numpy as np

from . import build as _build

INF_DIST = 1999999999
_lib = None

_I32 = ctypes.c_int32
_P = ctypes.c_void_p


def lib():
    global _lib
    if _lib is None:
        path = _build.build_oracle()
        L = ctypes.CDLL(path)
        L.orc_bellman_ford.restype = ctypes.c_int
        L.orc_bellman_ford.argtypes = [_I32, _P, _P, _P, _P, _P, _I32]
        L.orc_dijkstra.restype = None
        L.orc_dijkstra.argtypes = [_I32, _P, _P, _P, _I32, _P, _P, _P]
        L.orc_sssp_seeded.restype = ctypes.c_int
        L.orc_sssp_seeded.argtypes = [_I32, _P, _P, _P, _I32, _I32, _P, _P, _P]
        for name in ("orc_ppr_push_f64", "orc_ppr_push_f32"):
            fn = getattr(L, name)
            fn.restype = ctypes.c_int
            fn.argtypes = [_I32, _P, _P, _P, _I32, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                           ctypes.c_double, _I32, _I32, _I32, _I32, _P, _P, _P, _P, _P]
        L.orc_sssp_certificate.restype = ctypes.c_int64
        L.orc_sssp_certificate.argtypes = [_I32, _P, _P, _P, _I32, _P, _I32, _P, _P, _P,
                                           ctypes.POINTER(ctypes.c_int32)]
        L.orc_batch.restype = ctypes.c_int64
        L.orc_batch.argtypes = [ctypes.c_int, _I32, _P, _P, _P, _P, _I32, _P, _P, _P, _P, ctypes.c_double,
                                ctypes.c_double, _I32, _I32, _P, _P, _P, _P]
        L.orc_rmat_write.restype = ctypes.c_int
        L.orc_rmat_write.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint64, _I32, _I32,
                                     ctypes.c_double, ctypes.c_double, ctypes.c_double]
        L.orc_prune_sssp.restype = ctypes.c_int
        L.orc_prune_sssp.argtypes = [ctypes.c_char_p]
        L.orc_prune_ppr.restype = ctypes.c_int
        L.orc_prune_ppr.argtypes = [ctypes.c_char_p, ctypes.c_double]
        L.orc_prune_depth.restype = ctypes.c_int
        L.orc_prune_depth.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_double, _P]
        L.orc_prune_ppr_speculative.restype = ctypes.c_int
        L.orc_prune_ppr_speculative.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_int32, ctypes.c_char_p, _P]
        L.orc_prune_speculative.restype = ctypes.c_int
        L.orc_prune_speculative.argtypes = [ctypes.c_char_p, ctypes.c_int, ctypes.c_double, ctypes.c_int32,
                                            ctypes.c_char_p, _P]
        _lib = L
    return _lib


def _c(a, dtype):
    return np.ascontiguousarray(a, dtype=dtype)


def _p(a):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)


def load_dataset(dir, variant="origin"):
    """Arrays of <dir>/<variant>/ as numpy (missing files are left out)."""
    d = os.path.join(dir, variant)
    out = {}
    floats = {"flist"} | ({"wlist", "hwlist"} if variant == "ppr" else set())
    for name in ("vlist", "elist", "wlist", "flist", "hvlist", "helist", "hwlist", "hvmap"):
        p = os.path.join(d, name + ".bin")
        if os.path.exists(p):
            out[name] = np.fromfile(p, dtype=np.float32 if name in floats else np.int32)
    return out


def bellman_ford(row, col, w, dist, frontier):
    """Reference CPU Bellman-Ford (src/sssp/base-perk/SSSP.cpp:88-119); dist updated in place."""
    row, col, w = _c(row, np.int32), _c(col, np.int32), _c(w, np.int32)
    fr = _c(frontier, np.int32)
    assert dist.dtype == np.int32 and dist.flags.c_contiguous
    return lib().orc_bellman_ford(len(row) - 1, _p(row), _p(col), _p(w), _p(dist), _p(fr), len(fr))


def dijkstra(row, col, w, init_v, init_d):
    row, col, w = _c(row, np.int32), _c(col, np.int32), _c(w, np.int32)
    iv, idd = _c(init_v, np.int32), _c(init_d, np.int32)
    dist = np.empty(len(row) - 1, dtype=np.int32)
    lib().orc_dijkstra(len(row) - 1, _p(row), _p(col), _p(w), len(iv), _p(iv), _p(idd), _p(dist))
    return dist


def sssp_seeded(row, col, w, source, seed_v=(), seed_w=()):
    row, col, w = _c(row, np.int32), _c(col, np.int32), _c(w, np.int32)
    sv, sw = _c(seed_v, np.int32), _c(seed_w, np.int32)
    dist = np.empty(len(row) - 1, dtype=np.int32)
    rounds = lib().orc_sssp_seeded(len(row) - 1, _p(row), _p(col), _p(w), source, len(sv),
                                   _p(sv) if len(sv) else None, _p(sw) if len(sw) else None, _p(dist))
    return dist, rounds


def ppr_push(row, col, f, source, alpha, rmax, r0=1.0, pr0=None, max_iter=500, seeded=False,
             seed_v=(), seed_w=(), dtype=np.float64, degree_scaled=False, params_f32=True):
    """BSP forward push restating calcuatePPR; returns (pr, res, rounds, counters).

    The reference holds alpha, rmax and the start values as ValueType = float
    (src/ppr/purn/Main.cu:66-67, src/ppr/w-purn-perk/PPR.cpp:21); with params_f32 they
    are rounded to float32 first, so an FP64 run differs from an FP32 one only in its
    arithmetic, not in its threshold (double 1e-7 and float 1e-7 differ by 1.2e-15)."""
    row, col, f = _c(row, np.int32), _c(col, np.int32), _c(f, np.float32)
    sv, sw = _c(seed_v, np.int32), _c(seed_w, np.float32)
    V = len(row) - 1
    if pr0 is None:
        pr0 = alpha * r0
    if params_f32:
        alpha, rmax, r0, pr0 = (float(np.float32(x)) for x in (alpha, rmax, r0, pr0))
    pr = np.empty(V, dtype=dtype)
    res = np.empty(V, dtype=dtype)
    cnt = np.zeros(3, dtype=np.int64)
    fn = lib().orc_ppr_push_f64 if dtype == np.float64 else lib().orc_ppr_push_f32
    rounds = fn(V, _p(row), _p(col), _p(f), source, alpha, rmax, r0, pr0, max_iter, int(seeded),
                int(degree_scaled), len(sv), _p(sv) if len(sv) else None, _p(sw) if len(sw) else None,
                _p(pr), _p(res), _p(cnt))
    return pr, res, rounds, cnt


def sssp_certificate(row, col, w, dist, sources, seed_v=(), seed_w=()):
    """Check a distance vector against the Bellman conditions (orc_sssp_certificate);
    returns (number of violating vertices, first violating vertex or -1)."""
    row, col, w = _c(row, np.int32), _c(col, np.int32), _c(w, np.int32)
    src, sv, sw = _c(sources, np.int32), _c(seed_v, np.int32), _c(seed_w, np.int32)
    d = _c(dist, np.int32)
    bv = ctypes.c_int32()
    bad = lib().orc_sssp_certificate(len(row) - 1, _p(row), _p(col), _p(w), len(src), _p(src), len(sv),
                                     _p(sv) if len(sv) else None, _p(sw) if len(sw) else None, _p(d),
                                     ctypes.byref(bv))
    return int(bad), int(bv.value)


def batch(kind, row, col, w, f, sources, alpha=0.15, rmax=1e-7, max_iter=500, threads=1,
          keep=False, seeds=None, f64=False):
    """Independent queries on `threads` host threads (CPU baseline, parallel checks).
    kind 'sssp' (reference CPU Bellman-Ford) or 'ppr' (BSP push, float; double with
    f64).  seeds = (offsets[n+1], vertices, weights) gives each query its first hop
    (sssp-purn / ppr-purn), see query_seeds.  Returns (edges, outputs-or-None); the PPR
    outputs in double are (pr, res)."""
    row, col = _c(row, np.int32), _c(col, np.int32)
    w = None if w is None else _c(w, np.int32)
    f = None if f is None else _c(f, np.float32)
    src = _c(sources, np.int32)
    V = len(row) - 1
    k = 0 if kind == "sssp" else (2 if f64 else 1)
    so = sv = sw = None
    if seeds is not None:
        so, sv = _c(seeds[0], np.int32), _c(seeds[1], np.int32)
        sw = _c(seeds[2], np.int32 if k == 0 else np.float32)
        assert len(so) == len(src) + 1
    # the reference holds alpha and rmax as float (ppr_push's params_f32)
    alpha, rmax = float(np.float32(alpha)), float(np.float32(rmax))
    dist = pr = pr64 = res64 = None
    if keep:
        if k == 0:
            dist = np.empty((len(src), V), dtype=np.int32)
        elif k == 1:
            pr = np.empty((len(src), V), dtype=np.float32)
        else:
            pr64 = np.empty((len(src), V), dtype=np.float64)
            res64 = np.empty((len(src), V), dtype=np.float64)
    edges = lib().orc_batch(k, V, _p(row), _p(col), _p(w), _p(f), len(src), _p(src), _p(so), _p(sv), _p(sw),
                            alpha, rmax, max_iter, threads, _p(dist), _p(pr), _p(pr64), _p(res64))
    out = dist if k == 0 else (pr if k == 1 else (pr64, res64))
    return edges, (out if keep else None)


def query_seeds(ds, sources, kind):
    """First-hop seeds of each source as (offsets, vertices, weights).
    kind 'sssp': the source's own pruned record, found through the record->vertex
    sidecar (EXACT mode; sources without a record get none).  kind 'ppr': the source's
    record (hvlist indexed by vertex, src/ppr/purn/Main.cu:78-86) followed by its kept
    out-edges (:87-93)."""
    hv, he, hw = ds["hvlist"], ds["helist"], ds["hwlist"]
    rec_of = None
    if kind == "sssp":
        rec_of = np.full(len(ds["vlist"]) - 1, -1, dtype=np.int64)
        rec_of[ds["hvmap"]] = np.arange(len(ds["hvmap"]))
    off, vs, ws = [0], [], []
    for s in np.asarray(sources, dtype=np.int64):
        if kind == "sssp":
            r = rec_of[s]
            sv = he[hv[r]:hv[r + 1]] if r >= 0 else he[:0]
            sw = hw[hv[r]:hv[r + 1]] if r >= 0 else hw[:0]
        else:
            vl = ds["vlist"]
            sv = np.concatenate([he[hv[s]:hv[s + 1]], ds["elist"][vl[s]:vl[s + 1]]])
            sw = np.concatenate([hw[hv[s]:hv[s + 1]], ds["wlist"][vl[s]:vl[s + 1]]])
        vs.append(sv)
        ws.append(sw)
        off.append(off[-1] + len(sv))
    wdt = np.int32 if kind == "sssp" else np.float32
    v = np.concatenate(vs).astype(np.int32) if vs else np.zeros(0, np.int32)
    w = np.concatenate(ws).astype(wdt) if ws else np.zeros(0, wdt)
    return np.asarray(off, dtype=np.int32), v, w


def rmat_write(dir, scale, edge_factor, seed, wmin=1, wmax=100, a=0.57, b=0.19, c=0.19):
    """Seeded R-MAT graph in the origin/ layout (oracle/ingest.c orc_rmat_write)."""
    rc = lib().orc_rmat_write(os.fsencode(dir), scale, edge_factor, seed, wmin, wmax, a, b, c)
    if rc:
        raise RuntimeError("orc_rmat_write failed: %d" % rc)


def prune_sssp(dir):
    """purn-sssp restated (oracle/ingest.c orc_prune_sssp), plus sssp/hvmap.bin."""
    rc = lib().orc_prune_sssp(os.fsencode(dir))
    if rc:
        raise RuntimeError("orc_prune_sssp failed: %d" % rc)


def prune_ppr(dir, alpha=None):
    """purn-ppr restated (oracle/ingest.c orc_prune_ppr); alpha None keeps the
    reference's baked 0.8, else folded edges carry 1 - alpha."""
    rc = lib().orc_prune_ppr(os.fsencode(dir), 0.8 if alpha is None else 1.0 - alpha)
    if rc:
        raise RuntimeError("orc_prune_ppr failed: %d" % rc)


def prune_depth(dir, kind, alpha=None):
    """Run a pruner (kind "sssp" or "ppr") with the dependency analysis of its visiting
    order (oracle/ingest.c orc_prune_depth); writes the same outputs as prune_sssp /
    prune_ppr.  Returns the visits, the visits that moved edges, the visiting decisions,
    the depth (the longest chain of dependent operations, decisions included, and of
    pruning visits alone), the widest level, and the visits in levels of >= 32 and
    >= 1024 visits."""
    st = np.zeros(8, np.int64)
    keep = 0.8 if alpha is None else 1.0 - alpha
    rc = lib().orc_prune_depth(os.fsencode(dir), 1 if kind == "ppr" else 0, keep, st.ctypes.data)
    if rc:
        raise RuntimeError("orc_prune_depth failed: %d" % rc)
    keys = ("visits", "removing", "decisions", "depth", "visit_depth", "widest", "in_levels_ge32",
            "in_levels_ge1024")
    return {k: int(x) for k, x in zip(keys, st)}


def prune_speculative(dir, kind, alpha=None, window=1024, sub=None):
    """Either pruner's steps (kind "sssp" or "ppr") in rounds of the device pruners'
    reservation-based schedule over a window of `window` positions (oracle/ingest.c
    orc_prune_speculative); outputs in dir/<sub>/ (default <kind>_spec) in the sssp/ or ppr/
    layout.  Returns the rounds, the committed positions and the largest round."""
    st = np.zeros(3, np.int64)
    keep = 0.8 if alpha is None else 1.0 - alpha
    sub = sub or kind + "_spec"
    rc = lib().orc_prune_speculative(os.fsencode(dir), 1 if kind == "ppr" else 0, keep, int(window), sub.encode(),
                                     st.ctypes.data)
    if rc:
        raise RuntimeError("orc_prune_speculative failed: %d" % rc)
    return {"rounds": int(st[0]), "visits": int(st[1]), "widest": int(st[2])}


def prune_ppr_speculative(dir, alpha=None, window=1024, sub="ppr_spec"):
    """purn-ppr's visits run in rounds of a speculative, reservation-based schedule
    (oracle/ingest.c orc_prune_ppr_speculative); outputs in dir/<sub>/ in the ppr/
    layout.  Returns the rounds, the committed visits and the largest round."""
    st = np.zeros(3, np.int64)
    keep = 0.8 if alpha is None else 1.0 - alpha
    rc = lib().orc_prune_ppr_speculative(os.fsencode(dir), keep, int(window), sub.encode(), st.ctypes.data)
    if rc:
        raise RuntimeError("orc_prune_ppr_speculative failed: %d" % rc)
    return {"rounds": int(st[0]), "visits": int(st[1]), "widest": int(st[2])}


def adsorption_labels(row, col, f, seeds, p_inj, p_cont, iterations):
    """FP64 label propagation Y <- p_inj*I + p_cont * (A^T Y), A[u][v] = f(u,v), from
    Y = I (I[seed_l][l] = 1), with numpy/scipy."""
    import scipy.sparse as sp

    V = len(row) - 1
    L = len(seeds)
    A = sp.csr_matrix((np.asarray(f, dtype=np.float64), np.asarray(col), np.asarray(row)), shape=(V, V))
    AT = A.T.tocsr()
    I = np.zeros((V, L))
    for l, v in enumerate(seeds):
        I[v, l] += 1.0
    Y = I.copy()
    pi = np.asarray(p_inj, dtype=np.float64)[:, None]
    pc = np.asarray(p_cont, dtype=np.float64)[:, None]
    for _ in range(iterations):
        Y = pi * I + pc * (AT @ Y)
    return Y
