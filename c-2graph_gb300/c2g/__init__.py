"""Python host binding of the C^2graph GB300 library (ctypes over include/c2graph.h).

The library is the product; this module only marshals arguments.  It mirrors the
reference's programs: ``Graph.load(dir, "origin"|"sssp"|"ppr")`` reads the reference's
binary dataset layout, ``Graph.sssp`` / ``Graph.ppr`` run the sssp-base / sssp-purn /
ppr-base / ppr-purn traversals, ``prune_sssp`` / ``prune_ppr`` are purn-sssp /
purn-ppr, and ``rmat_write`` writes a synthetic origin/ dataset.

Importing never compiles anything; ``build()`` (the package's build.py) does.  A
missing library raises ``LibraryMissing``: there is no fallback implementation.
"""
import ctypes
import os

import numpy as np

PKG_DIR = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_PATH = os.path.join(PKG_DIR, "lib", "libc2graph.so")
BIN_DIR = os.path.join(PKG_DIR, "bin")
INCLUDE = os.path.join(os.path.dirname(PKG_DIR), "include", "c2graph.h")

INF_DIST = 1999999999

OK = 0
ERR_ARG, ERR_IO, ERR_FORMAT, ERR_CUDA, ERR_OOM = -1, -2, -3, -4, -5
ERR_RANGE, ERR_TIMEOUT, ERR_OVERFLOW, ERR_UNSUPPORTED, ERR_NODEVICE = -6, -7, -8, -9, -10
FLAG_BARRIER_TIMEOUT, FLAG_ITER_CAP, FLAG_QUEUE_OVERFLOW, FLAG_BOUNDS = 0x1, 0x2, 0x4, 0x8
NOALLOC_MAX_V, NOALLOC_MAX_E = 262144, 4194304  # size of c2g_sssp_noalloc's static scratch

VARIANTS = {"origin": 0, "sssp": 1, "ppr": 2}
SEEDS_COMPAT, SEEDS_EXACT = 0, 1


class LibraryMissing(RuntimeError):
    pass


class C2GError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("c2graph error %d: %s" % (code, msg))
        self.code = code


class Stats(ctypes.Structure):
    _fields_ = [("source", ctypes.c_int32), ("iterations", ctypes.c_int32),
                ("vertices_popped", ctypes.c_int64), ("edges_relaxed", ctypes.c_int64),
                ("touched", ctypes.c_int64), ("n_seeds", ctypes.c_int64),
                ("alg_bytes", ctypes.c_double), ("device_ms", ctypes.c_float),
                ("status_flags", ctypes.c_int32), ("reserved", ctypes.c_int32)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_ if k != "reserved"}


class ServerConfig(ctypes.Structure):
    _fields_ = [("max_batch", ctypes.c_int32), ("ads_iterations", ctypes.c_int32), ("alpha", ctypes.c_float),
                ("rmax", ctypes.c_float), ("hbm_budget_bytes", ctypes.c_int64), ("epoch_rounds", ctypes.c_int32),
                ("preempt_rounds", ctypes.c_int32)]


class Request(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int32), ("source", ctypes.c_int32), ("seeds", ctypes.c_void_p),
                ("out", ctypes.c_void_p)]


class ServerStats(ctypes.Structure):
    _fields_ = [("completed", ctypes.c_int64), ("batches", ctypes.c_int64 * 3), ("pending", ctypes.c_int64 * 3),
                ("admit_cap", ctypes.c_int64 * 3), ("max_batch", ctypes.c_int64), ("p50_ms", ctypes.c_double),
                ("p99_ms", ctypes.c_double), ("queries_per_s", ctypes.c_double), ("evictions", ctypes.c_int64)]


REQ_SSSP, REQ_PPR, REQ_ADSORPTION = 0, 1, 2


class PprParams(ctypes.Structure):
    _fields_ = [("alpha", ctypes.c_float), ("rmax", ctypes.c_float), ("r0", ctypes.c_float),
                ("pr0", ctypes.c_float), ("max_iter", ctypes.c_int32), ("seeded", ctypes.c_int32)]


_lib = None

_P = ctypes.c_void_p
_I32P = ctypes.POINTER(ctypes.c_int32)
_F32P = ctypes.POINTER(ctypes.c_float)

# name -> (restype, argtypes); every symbol include/c2graph.h declares.
SIGNATURES = {
    "c2g_abi_version": (ctypes.c_int, []),
    "c2g_last_error": (ctypes.c_char_p, []),
    "c2g_device_count": (ctypes.c_int, [_I32P]),
    "c2g_graph_load": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_P)]),
    "c2g_graph_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int32, ctypes.c_int64, _P, _P, _P, _P,
                                        ctypes.POINTER(_P)]),
    "c2g_graph_set_records": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P, _P, ctypes.c_int, _P]),
    "c2g_graph_free": (None, [_P]),
    "c2g_graph_info": (ctypes.c_int, [_P, _I32P, ctypes.POINTER(ctypes.c_int64), _I32P]),
    "c2g_graph_set_stream": (ctypes.c_int, [_P, _P]),
    "c2g_sssp_resolve_source": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int, ctypes.c_int, _I32P]),
    "c2g_sssp": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int,
                                ctypes.POINTER(Stats)]),
    "c2g_sssp_set_config": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32, ctypes.c_int32]),
    "c2g_sssp_noalloc": (ctypes.c_int, [_P, _P, ctypes.c_int32, ctypes.c_int64, ctypes.c_int32, _P, _P,
                                        ctypes.POINTER(Stats)]),
    "c2g_sssp_autotune": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_int, ctypes.c_int, ctypes.c_char_p,
                                         _I32P, _I32P]),
    "c2g_sssp_batch": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_int, ctypes.c_int, _P, ctypes.c_int,
                                      ctypes.c_int, ctypes.POINTER(Stats)]),
    "c2g_sssp_batch_set_tile": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    "c2g_sssp_batch_get_tile": (ctypes.c_int, [_P, _I32P, _I32P]),
    "c2g_sssp_batch_autotune": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_int, ctypes.c_int, ctypes.c_int32,
                                               ctypes.c_char_p, _I32P, _I32P]),
    "c2g_ppr": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(PprParams), _P, _P, ctypes.c_int,
                               ctypes.POINTER(Stats)]),
    "c2g_ppr_set_config": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    "c2g_ppr_batch_set_pull": (ctypes.c_int, [_P, ctypes.c_float]),
    "c2g_sssp_batch_set_pull": (ctypes.c_int, [_P, ctypes.c_float]),
    "c2g_sssp_batch_get_pull": (ctypes.c_int, [_P, ctypes.POINTER(ctypes.c_float)]),
    "c2g_ppr_batch_autotune": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.POINTER(PprParams), ctypes.c_int32,
                                              ctypes.c_char_p, _P]),
    "c2g_graph_set_watchdog": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.c_int32]),
    "c2g_graph_last_phases": (ctypes.c_int, [_P, _P]),
    "c2g_graph_last_rounds": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P, _P, _P, _I32P]),
    "c2g_ppr_default_params": (ctypes.c_int, [_P, ctypes.c_int, ctypes.POINTER(PprParams)]),
    "c2g_ppr_batch": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.POINTER(PprParams), _P, _P, ctypes.c_int,
                                     ctypes.c_int, ctypes.POINTER(Stats)]),
    "c2g_ppr_adjoint": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(PprParams), ctypes.c_int32, _P,
                                       ctypes.c_float, _P, _P, _P, ctypes.POINTER(ctypes.c_double), ctypes.c_int,
                                       ctypes.POINTER(Stats)]),
    "c2g_graph_set_weights": (ctypes.c_int, [_P, _P, ctypes.c_int]),
    "c2g_adsorption": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P, _P, _P, ctypes.c_int32, _P, ctypes.c_int,
                                      ctypes.POINTER(Stats)]),
    "c2g_server_create": (ctypes.c_int, [_P, _P, _P, _P, ctypes.POINTER(ServerConfig), ctypes.POINTER(_P)]),
    "c2g_server_submit": (ctypes.c_int, [_P, ctypes.POINTER(Request), ctypes.POINTER(ctypes.c_int64)]),
    "c2g_server_wait": (ctypes.c_int, [_P, ctypes.c_int64, ctypes.c_double, ctypes.POINTER(ctypes.c_int),
                                       ctypes.POINTER(ctypes.c_double)]),
    "c2g_server_get_stats": (ctypes.c_int, [_P, ctypes.POINTER(ServerStats)]),
    "c2g_server_destroy": (ctypes.c_int, [_P]),
    "c2g_session_create": (ctypes.c_int, [_P, ctypes.c_int, ctypes.c_int32, ctypes.POINTER(PprParams),
                                          ctypes.POINTER(_P)]),
    "c2g_session_admit": (ctypes.c_int, [_P, ctypes.c_int32, _I32P]),
    "c2g_session_step": (ctypes.c_int, [_P, ctypes.c_int32, _P, ctypes.c_int32, _I32P, ctypes.POINTER(Stats)]),
    "c2g_session_read": (ctypes.c_int, [_P, ctypes.c_int32, _P, _P, ctypes.c_int, ctypes.POINTER(Stats)]),
    "c2g_session_evict": (ctypes.c_int, [_P, ctypes.c_int32, ctypes.POINTER(_P)]),
    "c2g_session_resume": (ctypes.c_int, [_P, _P, _I32P]),
    "c2g_snapshot_free": (None, [_P]),
    "c2g_session_slot": (ctypes.c_int, [_P, ctypes.c_int32, _I32P, _I32P, _I32P]),
    "c2g_session_free": (None, [_P]),
    "c2g_rmat_write": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                      ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                      ctypes.c_double]),
    "c2g_rmat_write_gpu": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.c_int, ctypes.c_uint64,
                                          ctypes.c_int32, ctypes.c_int32, ctypes.c_double, ctypes.c_double,
                                          ctypes.c_double, ctypes.c_int]),
    "c2g_prune_sssp": (ctypes.c_int, [ctypes.c_char_p]),
    "c2g_convert_text": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(ctypes.c_int64),
                                        ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]),
    "c2g_prune_ppr": (ctypes.c_int, [ctypes.c_char_p]),
    "c2g_prune_ppr_alpha": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_double]),
    "c2g_prune_ppr_device": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_double, ctypes.c_int,
                                            ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_int32),
                                            ctypes.c_void_p]),
    "c2g_prune_sssp_device": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int, ctypes.POINTER(ctypes.c_float),
                                             ctypes.POINTER(ctypes.c_int32), ctypes.c_void_p]),
}


def lib():
    """Load libc2graph.so (raises LibraryMissing when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.isfile(LIB_PATH):
            raise LibraryMissing("libc2graph.so not built: run __graft_entry__.build() "
                                 "(expected at %s)" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def _check(rc):
    if rc != OK:
        msg = lib().c2g_last_error()
        raise C2GError(rc, msg.decode() if msg else "")
    return rc


def _ptr(a):
    return ctypes.c_void_p(a.ctypes.data) if a is not None else None


def device_count():
    n = ctypes.c_int32(0)
    _check(lib().c2g_device_count(ctypes.byref(n)))
    return n.value


def rmat_write(dir, scale, edge_factor, seed, wmin=1, wmax=100, a=0.57, b=0.19, c=0.19, gpu=False, device=0):
    """Seeded R-MAT graph in the origin/ layout; gpu=True builds it on the device (same bytes)."""
    if gpu:
        _check(lib().c2g_rmat_write_gpu(os.fsencode(dir), scale, edge_factor, seed, wmin, wmax, a, b, c, device))
    else:
        _check(lib().c2g_rmat_write(os.fsencode(dir), scale, edge_factor, seed, wmin, wmax, a, b, c))


def convert_text(text_path, dir):
    """convert2binary: a text edge list into dir/origin/.  Returns (max vertex, V, E)."""
    mv, v, e = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
    _check(lib().c2g_convert_text(os.fsencode(text_path), os.fsencode(dir), ctypes.byref(mv), ctypes.byref(v),
                                  ctypes.byref(e)))
    return int(mv.value), int(v.value), int(e.value)


def prune_sssp(dir):
    _check(lib().c2g_prune_sssp(os.fsencode(dir)))


def prune_ppr(dir, alpha=None):
    """purn-ppr; with alpha, folded edges carry 1 - alpha instead of the baked 0.8."""
    if alpha is None:
        _check(lib().c2g_prune_ppr(os.fsencode(dir)))
    else:
        _check(lib().c2g_prune_ppr_alpha(os.fsencode(dir), float(alpha)))


def prune_ppr_device(dir, alpha=0.2, device=0, phases=False):
    """purn-ppr on the GPU (same files as prune_ppr(dir, alpha)).  Returns (kernel ms, rounds),
    and with phases=True also the kernel ms of the rounds' plan, check, commit and copy
    phases."""
    ms = ctypes.c_float(0.0)
    rounds = ctypes.c_int32(0)
    ph = np.zeros(4, np.int64)
    _check(lib().c2g_prune_ppr_device(os.fsencode(dir), float(alpha), int(device), ctypes.byref(ms),
                                      ctypes.byref(rounds), ph.ctypes.data))
    if phases:
        return float(ms.value), int(rounds.value), [float(x) / 1e6 for x in ph]
    return float(ms.value), int(rounds.value)


def prune_sssp_device(dir, device=0, phases=False):
    """purn-sssp on the GPU (same files as prune_sssp(dir), hvmap.bin included).  Returns
    (kernel ms, rounds), and with phases=True also the phases' kernel ms."""
    ms = ctypes.c_float(0.0)
    rounds = ctypes.c_int32(0)
    ph = np.zeros(4, np.int64)
    _check(lib().c2g_prune_sssp_device(os.fsencode(dir), int(device), ctypes.byref(ms), ctypes.byref(rounds),
                                       ph.ctypes.data))
    if phases:
        return float(ms.value), int(rounds.value), [float(x) / 1e6 for x in ph]
    return float(ms.value), int(rounds.value)


def read_array(path, dtype=np.int32):
    """Read a reference binary array (raw 4-byte elements, no header)."""
    return np.fromfile(path, dtype=dtype)


class Graph:
    """A device-resident graph handle."""

    def __init__(self, handle):
        self._h = handle
        V = ctypes.c_int32()
        E = ctypes.c_int64()
        R = ctypes.c_int32()
        _check(lib().c2g_graph_info(self._h, ctypes.byref(V), ctypes.byref(E), ctypes.byref(R)))
        self.V, self.E, self.R = V.value, E.value, R.value

    @classmethod
    def load(cls, dir, variant="origin", device=0):
        h = ctypes.c_void_p()
        _check(lib().c2g_graph_load(os.fsencode(dir), VARIANTS[variant], device, ctypes.byref(h)))
        return cls(h)

    @classmethod
    def create(cls, vlist, elist, wlist=None, flist=None, device=0):
        vlist = np.ascontiguousarray(vlist, dtype=np.int32)
        elist = np.ascontiguousarray(elist, dtype=np.int32)
        wlist = None if wlist is None else np.ascontiguousarray(wlist, dtype=np.int32)
        flist = None if flist is None else np.ascontiguousarray(flist, dtype=np.float32)
        h = ctypes.c_void_p()
        _check(lib().c2g_graph_create(device, len(vlist) - 1, len(elist), _ptr(vlist), _ptr(elist),
                                      _ptr(wlist), _ptr(flist), ctypes.byref(h)))
        return cls(h)

    def set_records(self, hvlist, helist, hwlist, record_vertex=None):
        hvlist = np.ascontiguousarray(hvlist, dtype=np.int32)
        helist = np.ascontiguousarray(helist, dtype=np.int32)
        is_float = np.asarray(hwlist).dtype.kind == "f"
        hwlist = np.ascontiguousarray(hwlist, dtype=np.float32 if is_float else np.int32)
        rv = None if record_vertex is None else np.ascontiguousarray(record_vertex, dtype=np.int32)
        _check(lib().c2g_graph_set_records(self._h, len(hvlist) - 1, _ptr(hvlist), _ptr(helist),
                                           _ptr(hwlist), int(is_float), _ptr(rv)))
        self.R = len(hvlist) - 1

    def close(self):
        if self._h:
            lib().c2g_graph_free(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def set_stream(self, stream_ptr):
        _check(lib().c2g_graph_set_stream(self._h, ctypes.c_void_p(stream_ptr)))

    def sssp_config(self, delta=0, tile=256, max_iter=1 << 20):
        _check(lib().c2g_sssp_set_config(self._h, delta, tile, max_iter))

    def sssp_autotune(self, sources, seeds=False, mode=SEEDS_COMPAT, json_path=None):
        """Pick the fastest (delta, tile) for this graph; returns (delta, tile)."""
        src = np.ascontiguousarray(sources, dtype=np.int32)
        bd, bt = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().c2g_sssp_autotune(self._h, len(src), _ptr(src), int(seeds), mode,
                                       os.fsencode(json_path) if json_path else None, ctypes.byref(bd),
                                       ctypes.byref(bt)))
        return bd.value, bt.value

    def sssp_batch_tile(self, big_steps=512, min_tiles_per_warp=16):
        """Expansion tiles of the batched SSSP (see c2g_sssp_batch_set_tile)."""
        _check(lib().c2g_sssp_batch_set_tile(self._h, big_steps, min_tiles_per_warp))

    def sssp_batch_pull(self, frac=0.5):
        """Batched SSSP rounds with more than frac * E * Q (query, edge) relaxations pull over
        the reverse CSR (Q: query slots; frac < 0: expand only; 0: every round)."""
        _check(lib().c2g_sssp_batch_set_pull(self._h, float(frac)))

    def sssp_batch_pull_frac(self):
        """The batched SSSP's current pull fraction (c2g_sssp_batch_get_pull)."""
        f = ctypes.c_float()
        _check(lib().c2g_sssp_batch_get_pull(self._h, ctypes.byref(f)))
        return f.value

    def sssp_batch_autotune(self, sources, seeds=False, mode=SEEDS_COMPAT, reps=1, json_path=None):
        """Time the batched SSSP's tile candidates on this batch, apply the fastest valid
        one and return it as (big_steps, min_tiles_per_warp)."""
        src = np.ascontiguousarray(sources, dtype=np.int32)
        bb, bm = ctypes.c_int32(), ctypes.c_int32()
        _check(lib().c2g_sssp_batch_autotune(self._h, len(src), _ptr(src), int(seeds), mode, int(reps),
                                             os.fsencode(json_path) if json_path else None, ctypes.byref(bb),
                                             ctypes.byref(bm)))
        return bb.value, bm.value

    def resolve_source(self, source, pruned=False, mode=SEEDS_COMPAT):
        out = ctypes.c_int32()
        _check(lib().c2g_sssp_resolve_source(self._h, source, int(pruned), mode, ctypes.byref(out)))
        return out.value

    def sssp(self, source, seeds=False, mode=SEEDS_COMPAT, out=None, out_ptr=None):
        """Distances as an int32 numpy array (or into device memory at out_ptr)."""
        st = Stats()
        if out_ptr is not None:
            _check(lib().c2g_sssp(self._h, source, int(seeds), mode, ctypes.c_void_p(out_ptr), 1,
                                  ctypes.byref(st)))
            return None, st
        dist = out if out is not None else np.empty(self.V, dtype=np.int32)
        _check(lib().c2g_sssp(self._h, source, int(seeds), mode, _ptr(dist), 0, ctypes.byref(st)))
        return dist, st

    def sssp_batch(self, sources, seeds=False, mode=SEEDS_COMPAT, out=None, out_ptr=None, vertex_major=False):
        """Batched SSSP: (n, V) int32 distances (query-major), or into device memory."""
        src = np.ascontiguousarray(sources, dtype=np.int32)
        st = Stats()
        layout = 1 if vertex_major else 0
        if out_ptr is not None:
            _check(lib().c2g_sssp_batch(self._h, len(src), _ptr(src), int(seeds), mode, ctypes.c_void_p(out_ptr), 1,
                                        layout, ctypes.byref(st)))
            return None, st
        dist = out if out is not None else np.empty((len(src), self.V) if not vertex_major else (self.V, len(src)),
                                                    dtype=np.int32)
        _check(lib().c2g_sssp_batch(self._h, len(src), _ptr(src), int(seeds), mode, _ptr(dist), 0, layout,
                                    ctypes.byref(st)))
        return dist, st

    def last_phases(self):
        """(init, frontier build/apply, expand/push, reserved) ms of the last launch."""
        out = np.zeros(4, dtype=np.float64)
        _check(lib().c2g_graph_last_phases(self._h, _ptr(out)))
        return tuple(float(x) for x in out)

    def last_rounds(self, first_phase=False):
        """Per-round (ms, work units, pull) of the last batched launch on this handle;
        with first_phase, (ms, first-phase ms, work units, pull)."""
        ms = np.zeros(1024, dtype=np.float64)
        first = np.zeros(1024, dtype=np.float64)
        work = np.zeros(1024, dtype=np.int64)
        shape = np.zeros(1024, dtype=np.int32)
        n = ctypes.c_int32()
        _check(lib().c2g_graph_last_rounds(self._h, 1024, _ptr(ms), _ptr(first), _ptr(work), _ptr(shape),
                                           ctypes.byref(n)))
        k = n.value
        return (ms[:k], first[:k], work[:k], shape[:k]) if first_phase else (ms[:k], work[:k], shape[:k])

    def watchdog(self, barrier_timeout_ms=0, stall_next_sssp=False):
        _check(lib().c2g_graph_set_watchdog(self._h, barrier_timeout_ms, int(bool(stall_next_sssp))))

    def ppr_config(self, pull_div=0, dense_div=16):
        _check(lib().c2g_ppr_set_config(self._h, pull_div, dense_div))

    def ppr_batch_pull(self, ratio=8.0):
        """Batched rounds with more than ratio * E pushes pull over the reverse CSR
        (ratio < 0: push only; 0: every round)."""
        _check(lib().c2g_ppr_batch_set_pull(self._h, float(ratio)))

    def ppr_batch_autotune(self, sources, params, reps=1, json_path=None):
        """Time the pull ratios on this batch, apply the fastest valid one and return it."""
        src = np.ascontiguousarray(sources, dtype=np.int32)
        best = ctypes.c_float(0.0)
        _check(lib().c2g_ppr_batch_autotune(self._h, len(src), _ptr(src), ctypes.byref(params), int(reps),
                                            json_path.encode() if json_path else None, ctypes.byref(best)))
        return float(best.value)

    def ppr_params(self, adsorption=False, **kw):
        p = PprParams()
        _check(lib().c2g_ppr_default_params(self._h, int(adsorption), ctypes.byref(p)))
        for k, v in kw.items():
            setattr(p, k, v)
        return p

    def ppr(self, source, params=None, pr_ptr=None, res_ptr=None, **kw):
        """(pr, res, stats) as float32 numpy arrays (or into device memory)."""
        p = params if params is not None else self.ppr_params(**kw)
        st = Stats()
        if pr_ptr is not None:
            _check(lib().c2g_ppr(self._h, source, ctypes.byref(p), ctypes.c_void_p(pr_ptr),
                                 ctypes.c_void_p(res_ptr) if res_ptr else None, 1, ctypes.byref(st)))
            return None, None, st
        pr = np.empty(self.V, dtype=np.float32)
        res = np.empty(self.V, dtype=np.float32)
        _check(lib().c2g_ppr(self._h, source, ctypes.byref(p), _ptr(pr), _ptr(res), 0, ctypes.byref(st)))
        return pr, res, st

    def ppr_batch(self, sources, params=None, pr_ptr=None, res_ptr=None, want_res=True, vertex_major=False, **kw):
        """Batched push: (pr, res, stats) with (n, V) float32 arrays (query-major)."""
        src = np.ascontiguousarray(sources, dtype=np.int32)
        p = params if params is not None else self.ppr_params(**kw)
        st = Stats()
        layout = 1 if vertex_major else 0
        if pr_ptr is not None:
            _check(lib().c2g_ppr_batch(self._h, len(src), _ptr(src), ctypes.byref(p), ctypes.c_void_p(pr_ptr),
                                       ctypes.c_void_p(res_ptr) if res_ptr else None, 1, layout, ctypes.byref(st)))
            return None, None, st
        shape = (len(src), self.V) if not vertex_major else (self.V, len(src))
        pr = np.empty(shape, dtype=np.float32)
        res = np.empty(shape, dtype=np.float32) if want_res else None
        _check(lib().c2g_ppr_batch(self._h, len(src), _ptr(src), ctypes.byref(p), _ptr(pr), _ptr(res), 0, layout,
                                   ctypes.byref(st)))
        return pr, res, st

    def set_weights(self, flist=None, ptr=None):
        """Replace the float edge weights (host array, or a device pointer)."""
        if ptr is not None:
            _check(lib().c2g_graph_set_weights(self._h, ctypes.c_void_p(ptr), 1))
        else:
            f = np.ascontiguousarray(flist, dtype=np.float32)
            _check(lib().c2g_graph_set_weights(self._h, _ptr(f), 0))

    def ppr_adjoint(self, source, targets, params=None, rmax_backward=1e-8, **kw):
        """(grad[E], pi[V], lambda[V], loss, stats) of L = sum_t pi_source(t)."""
        p = params if params is not None else self.ppr_params(**kw)
        t = np.ascontiguousarray(targets, dtype=np.int32)
        grad = np.empty(self.E, dtype=np.float32)
        pi = np.empty(self.V, dtype=np.float32)
        lam = np.empty(self.V, dtype=np.float32)
        loss = ctypes.c_double()
        st = Stats()
        _check(lib().c2g_ppr_adjoint(self._h, source, ctypes.byref(p), len(t), _ptr(t), rmax_backward, _ptr(grad),
                                     _ptr(pi), _ptr(lam), ctypes.byref(loss), 0, ctypes.byref(st)))
        return grad, pi, lam, loss.value, st

    def adsorption_device(self, seeds, p_inj_ptr, p_cont_ptr, p_abnd_ptr, Y_ptr, iterations=30):
        """Label propagation with p_* and Y[V,16] in device memory (pointers); returns stats."""
        sv = np.ascontiguousarray(seeds, dtype=np.int32)
        st = Stats()
        _check(lib().c2g_adsorption(self._h, len(sv), _ptr(sv), ctypes.c_void_p(p_inj_ptr), ctypes.c_void_p(p_cont_ptr),
                                    ctypes.c_void_p(p_abnd_ptr), iterations, ctypes.c_void_p(Y_ptr), 1,
                                    ctypes.byref(st)))
        return st

    def adsorption(self, seeds, p_inj, p_cont, p_abnd, iterations=30):
        """Label propagation: (Y[V,16] float32, stats)."""
        sv = np.ascontiguousarray(seeds, dtype=np.int32)
        pi = np.ascontiguousarray(p_inj, dtype=np.float32)
        pc = np.ascontiguousarray(p_cont, dtype=np.float32)
        pa = np.ascontiguousarray(p_abnd, dtype=np.float32)
        Y = np.empty((self.V, 16), dtype=np.float32)
        st = Stats()
        _check(lib().c2g_adsorption(self._h, len(sv), _ptr(sv), _ptr(pi), _ptr(pc), _ptr(pa), iterations, _ptr(Y), 0,
                                    ctypes.byref(st)))
        return Y, st


class Session:
    """Resident batch of one query kind (c2g_session_*): admit sources into slots, run
    epochs, read finished results, evict running queries into snapshots and resume them."""

    def __init__(self, graph, kind, slots, params=None):
        self.graph = graph
        self.kind = kind
        self._h = _P()
        _check(lib().c2g_session_create(graph._h, kind, slots, ctypes.byref(params) if params is not None else None,
                                        ctypes.byref(self._h)))

    def admit(self, source):
        slot = ctypes.c_int32()
        _check(lib().c2g_session_admit(self._h, int(source), ctypes.byref(slot)))
        return slot.value

    def step(self, rounds=4):
        """One epoch; returns (finished slots, stats)."""
        fin = np.zeros(1024, dtype=np.int32)
        n = ctypes.c_int32()
        st = Stats()
        _check(lib().c2g_session_step(self._h, int(rounds), _ptr(fin), len(fin), ctypes.byref(n), ctypes.byref(st)))
        return fin[:n.value].tolist(), st

    def read(self, slot, want_res=False):
        """Result of a finished slot (SSSP int32 distances; PPR (pr, res)); frees it."""
        V = self.graph.V
        st = Stats()
        if self.kind == REQ_SSSP:
            out = np.empty(V, dtype=np.int32)
            _check(lib().c2g_session_read(self._h, slot, _ptr(out), None, 0, ctypes.byref(st)))
            return out, st
        pr = np.empty(V, dtype=np.float32)
        res = np.empty(V, dtype=np.float32) if want_res else None
        _check(lib().c2g_session_read(self._h, slot, _ptr(pr), _ptr(res), 0, ctypes.byref(st)))
        return (pr, res), st

    def evict(self, slot):
        snap = _P()
        _check(lib().c2g_session_evict(self._h, slot, ctypes.byref(snap)))
        return snap

    def resume(self, snap):
        slot = ctypes.c_int32()
        _check(lib().c2g_session_resume(self._h, snap, ctypes.byref(slot)))
        return slot.value

    def slot(self, slot):
        st, src, rounds = ctypes.c_int32(), ctypes.c_int32(), ctypes.c_int32()
        _check(lib().c2g_session_slot(self._h, slot, ctypes.byref(st), ctypes.byref(src), ctypes.byref(rounds)))
        return st.value, src.value, rounds.value

    def close(self):
        if self._h:
            lib().c2g_session_free(self._h)
            self._h = _P()

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


class Server:
    """Continuous-batching request loop over a device-resident graph."""

    def __init__(self, graph, max_batch=256, alpha=0.15, rmax=1e-7, ads_iterations=30, hbm_budget_bytes=0,
                 p_inj=None, p_cont=None, p_abnd=None, epoch_rounds=4, preempt_rounds=0):
        self.graph = graph
        cfg = ServerConfig(max_batch, ads_iterations, alpha, rmax, hbm_budget_bytes, epoch_rounds, preempt_rounds)
        self._p = [None if a is None else np.ascontiguousarray(a, dtype=np.float32) for a in (p_inj, p_cont, p_abnd)]
        h = ctypes.c_void_p()
        _check(lib().c2g_server_create(graph._h, *[_ptr(a) for a in self._p], ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        self._keep = {}

    def submit(self, kind, source=0, seeds=None, out=None):
        sv = None if seeds is None else np.ascontiguousarray(seeds, dtype=np.int32)
        req = Request(kind, source, _ptr(sv), _ptr(out))
        t = ctypes.c_int64()
        _check(lib().c2g_server_submit(self._h, ctypes.byref(req), ctypes.byref(t)))
        self._keep[t.value] = (sv, out)
        return t.value

    def wait(self, ticket, timeout=600.0):
        st = ctypes.c_int()
        lat = ctypes.c_double()
        _check(lib().c2g_server_wait(self._h, ticket, timeout, ctypes.byref(st), ctypes.byref(lat)))
        self._keep.pop(ticket, None)
        return st.value, lat.value

    def stats(self):
        s = ServerStats()
        _check(lib().c2g_server_get_stats(self._h, ctypes.byref(s)))
        return s

    def close(self):
        if self._h:
            lib().c2g_server_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()
