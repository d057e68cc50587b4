"""galp_gb300 -- GB300-native label propagation with galp's exact method-0 semantics.

Python mirror of the reference's propagator interface
(label_propagation/include/label_propagator.h:11-34):

    g = galp_gb300.load_graph("graph.bin")            # CSRGraph<int32,int64> (include/graph.h)
    p = galp_gb300.Propagator(g, method=0, policy=0)  # main.cu:139-207 factory
    f1, f2 = p.run(10)                                # LabelPropagator::run(niter)
    labels = p.get_labels()                           # LabelPropagator::get_labels()

Everything runs through the C ABI of lib/libgalp.so (include/galp.h).  There is no
CPU fallback: constructing a Propagator without the CUDA library or a GPU raises.
"""
from __future__ import annotations

import ctypes
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(_HERE, "lib")

GALP_MAX_ITERS = 64

ERRORS = {
    0: "ok", -1: "invalid argument", -2: "out of memory", -3: "CUDA error", -4: "device wait timed out",
    -5: "malformed graph", -6: "unsupported method/policy", -7: "no CUDA device",
    -8: "vertex degree exceeds the out-of-core batch buffer",
}


class GalpError(RuntimeError):
    def __init__(self, code: int, what: str = ""):
        self.code = code
        super().__init__(f"{what}: {ERRORS.get(code, 'error')} ({code})" if what else ERRORS.get(code, str(code)))


class _Csr(ctypes.Structure):
    _fields_ = [("neighbors", ctypes.c_void_p), ("offsets", ctypes.c_void_p),
                ("n", ctypes.c_int64), ("m", ctypes.c_int64)]


class Opts(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int32), ("policy", ctypes.c_int32), ("lfht_policy", ctypes.c_int32),
                ("buffer_pow", ctypes.c_int32), ("frontier", ctypes.c_int32), ("dispatch", ctypes.c_int32),
                ("device", ctypes.c_int32), ("early_exit", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("f1", ctypes.c_double), ("f2", ctypes.c_double), ("device_ms", ctypes.c_double),
                ("iters_run", ctypes.c_int32), ("err", ctypes.c_int32),
                ("updates", ctypes.c_int64 * GALP_MAX_ITERS), ("runs_last", ctypes.c_int64),
                ("h2d_bytes", ctypes.c_int64), ("d2h_bytes", ctypes.c_int64)]


class _GenGraph(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int64), ("m", ctypes.c_int64), ("offsets", ctypes.POINTER(ctypes.c_int64)),
                ("neighbors", ctypes.POINTER(ctypes.c_int32)), ("community", ctypes.POINTER(ctypes.c_int32))]


_lib = None
_gen = None


def lib_path(name: str) -> str:
    return os.path.join(LIB_DIR, name)


def load_library() -> ctypes.CDLL:
    """Load lib/libgalp.so (the CUDA library).  Raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    path = lib_path("libgalp.so")
    if not os.path.exists(path):
        raise RuntimeError(f"galp_gb300: CUDA library not built ({path}); run galp_gb300.build.build()")
    L = ctypes.CDLL(path)
    P = ctypes.c_void_p
    L.galp_default_opts.argtypes = [ctypes.POINTER(Opts)]
    L.galp_default_opts.restype = None
    L.galp_create.argtypes = [ctypes.POINTER(_Csr), ctypes.POINTER(Opts), ctypes.POINTER(P)]
    L.galp_create.restype = ctypes.c_int
    L.galp_run.argtypes = [P, ctypes.c_int32, ctypes.POINTER(Stats)]
    L.galp_run.restype = ctypes.c_int
    L.galp_enqueue.argtypes = [P, ctypes.c_int32]
    L.galp_enqueue.restype = ctypes.c_int
    L.galp_sync.argtypes = [P, ctypes.POINTER(Stats)]
    L.galp_sync.restype = ctypes.c_int
    L.galp_get_labels.argtypes = [P, P, ctypes.c_int64]
    L.galp_get_labels.restype = ctypes.c_int
    L.galp_destroy.argtypes = [P]
    L.galp_destroy.restype = None
    L.galp_strerror.argtypes = [ctypes.c_int]
    L.galp_strerror.restype = ctypes.c_char_p
    L.galp_set_stream.argtypes = [P, P]
    L.galp_set_stream.restype = ctypes.c_int
    L.galp_debug_resolve_rank.argtypes = [ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, P,
                                          ctypes.c_int32]
    L.galp_debug_resolve_rank.restype = ctypes.c_int32
    L.galp_batch_create.argtypes = [P, P, ctypes.c_int64, ctypes.c_int64, P, ctypes.c_int32, ctypes.POINTER(Opts),
                                    ctypes.POINTER(P)]
    L.galp_batch_create.restype = ctypes.c_int
    L.galp_batch_stats.argtypes = [P, ctypes.c_int32, ctypes.POINTER(Stats)]
    L.galp_batch_stats.restype = ctypes.c_int
    L.galp_batch_labels.argtypes = [P, ctypes.c_int32, P, ctypes.c_int64]
    L.galp_batch_labels.restype = ctypes.c_int
    L.galp_run_batch.argtypes = [P, ctypes.c_int32, ctypes.POINTER(Opts), ctypes.c_int32, P, P]
    L.galp_run_batch.restype = ctypes.c_int
    _lib = L
    return L


def load_generators() -> ctypes.CDLL:
    global _gen
    if _gen is not None:
        return _gen
    path = lib_path("libgalp_gen.so")
    if not os.path.exists(path):
        raise RuntimeError(f"galp_gb300: generator library not built ({path})")
    G = ctypes.CDLL(path)
    GP = ctypes.POINTER(_GenGraph)
    G.galp_gen_sbm.argtypes = [ctypes.c_void_p, ctypes.c_int32, ctypes.c_double, ctypes.c_double, ctypes.c_uint64]
    G.galp_gen_sbm.restype = GP
    G.galp_gen_rmat.argtypes = [ctypes.c_int32, ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                                ctypes.c_uint64]
    G.galp_gen_rmat.restype = GP
    G.galp_gen_lfr.argtypes = [ctypes.c_int64, ctypes.c_double, ctypes.c_double, ctypes.c_int64, ctypes.c_double,
                               ctypes.c_int64, ctypes.c_int64, ctypes.c_double, ctypes.c_uint64]
    G.galp_gen_lfr.restype = GP
    G.galp_graph_free.argtypes = [GP]
    G.galp_graph_free.restype = None
    G.galp_graph_write_bin.argtypes = [GP, ctypes.c_char_p]
    G.galp_graph_write_bin.restype = ctypes.c_int
    G.galp_graph_write_gt.argtypes = [GP, ctypes.c_char_p]
    G.galp_graph_write_gt.restype = ctypes.c_int
    _gen = G
    return G


@dataclass
class Graph:
    """CSR graph: offsets int64[n+1], neighbors int32[m]; community int32[n] or None."""
    offsets: np.ndarray
    neighbors: np.ndarray
    community: np.ndarray | None = None

    @property
    def n(self) -> int:
        return len(self.offsets) - 1

    @property
    def m(self) -> int:
        return len(self.neighbors)

    def degrees(self) -> np.ndarray:
        return np.diff(self.offsets)


def _take_generated(ptr) -> Graph:
    if not ptr:
        raise MemoryError("graph generation failed")
    g = ptr.contents
    n, m = g.n, g.m
    off = np.ctypeslib.as_array(g.offsets, (n + 1,)).copy()
    nbr = np.ctypeslib.as_array(g.neighbors, (max(m, 1),))[:m].copy()
    com = np.ctypeslib.as_array(g.community, (max(n, 1),))[:n].copy()
    load_generators().galp_graph_free(ptr)
    return Graph(off, nbr, com if (com >= 0).any() else None)


def generate_sbm(block_sizes, deg_in: float, deg_out: float, seed: int) -> Graph:
    bs = np.ascontiguousarray(block_sizes, dtype=np.int64)
    return _take_generated(load_generators().galp_gen_sbm(bs.ctypes.data, len(bs), deg_in, deg_out, seed))


def generate_rmat(scale: int, edge_factor: int, a=0.57, b=0.19, c=0.19, seed: int = 1) -> Graph:
    return _take_generated(load_generators().galp_gen_rmat(scale, edge_factor, a, b, c, seed))


def generate_lfr(n: int, tau1=2.5, kmean=20.0, kmax=1000, tau2=1.5, cmin=20, cmax=1000, mu=0.3,
                 seed: int = 1) -> Graph:
    return _take_generated(load_generators().galp_gen_lfr(n, tau1, kmean, kmax, tau2, cmin, cmax, mu, seed))


def default_opts(**kw) -> Opts:
    o = Opts()
    load_library().galp_default_opts(ctypes.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise TypeError(f"unknown option {k}")
        setattr(o, k, int(v))
    return o


def _check(rc: int, what: str) -> None:
    if rc != 0:
        raise GalpError(rc, what)


class Propagator:
    """GPU label propagator over a host CSR graph (LabelPropagator<int32,int64>)."""

    def __init__(self, graph: Graph, **opts):
        L = load_library()
        self.graph = graph
        self._off = np.ascontiguousarray(graph.offsets, dtype=np.int64)
        self._nbr = np.ascontiguousarray(graph.neighbors, dtype=np.int32)
        self._csr = _Csr(self._nbr.ctypes.data if len(self._nbr) else None, self._off.ctypes.data,
                         len(self._off) - 1, len(self._nbr))
        self.opts = default_opts(**opts)
        h = ctypes.c_void_p()
        _check(L.galp_create(ctypes.byref(self._csr), ctypes.byref(self.opts), ctypes.byref(h)), "galp_create")
        self._h = h
        self.stats = Stats()

    def run(self, niter: int = 10) -> tuple[float, float]:
        _check(load_library().galp_run(self._h, niter, ctypes.byref(self.stats)), "galp_run")
        return self.stats.f1, self.stats.f2

    def enqueue(self, niter: int) -> None:
        _check(load_library().galp_enqueue(self._h, niter), "galp_enqueue")

    def sync(self) -> Stats:
        _check(load_library().galp_sync(self._h, ctypes.byref(self.stats)), "galp_sync")
        return self.stats

    def set_stream(self, stream_ptr: int | None) -> None:
        _check(load_library().galp_set_stream(self._h, stream_ptr), "galp_set_stream")

    def get_labels(self) -> np.ndarray:
        out = np.empty(self.graph.n, dtype=np.int32)
        _check(load_library().galp_get_labels(self._h, out.ctypes.data if len(out) else None, len(out)),
               "galp_get_labels")
        return out

    @property
    def iters_run(self) -> int:
        return self.stats.iters_run

    @property
    def updates(self) -> list[int]:
        return list(self.stats.updates[: self.stats.iters_run])

    def close(self) -> None:
        if getattr(self, "_h", None):
            load_library().galp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()


class Batch:
    """Many independent graphs clustered together (include/galp.h galp_batch_create): each
    graph gets exactly the labels, iteration count and change counts of its own run.

    Either `graphs` (a list of Graph, concatenated here) or one concatenated CSR:
    `offsets` int64[n+1] and `neighbors` int32[m] with global IDs (numpy arrays, or
    integer device pointers together with n and m) and `graph_v0` int64[count+1]."""

    def __init__(self, graphs=None, *, offsets=None, neighbors=None, graph_v0=None, n=None, m=None, **opts):
        L = load_library()
        if graphs is not None:
            sizes = np.array([g.n for g in graphs], np.int64)
            graph_v0 = np.zeros(len(graphs) + 1, np.int64)
            graph_v0[1:] = np.cumsum(sizes)
            ecount = np.array([g.m for g in graphs], np.int64)
            e0 = np.zeros(len(graphs) + 1, np.int64)
            e0[1:] = np.cumsum(ecount)
            offsets = np.concatenate([np.asarray(g.offsets[:-1], np.int64) + e0[i] for i, g in enumerate(graphs)]
                                     + [np.array([e0[-1]], np.int64)])
            neighbors = np.concatenate([np.asarray(g.neighbors, np.int64) + graph_v0[i]
                                        for i, g in enumerate(graphs)]).astype(np.int32)
        self.graph_v0 = np.ascontiguousarray(graph_v0, np.int64)
        self.count = len(self.graph_v0) - 1
        if isinstance(offsets, int):
            off_p, nbr_p = offsets, neighbors
            self.n, self.m = int(n), int(m)
        else:
            self._off = np.ascontiguousarray(offsets, np.int64)
            self._nbr = np.ascontiguousarray(neighbors, np.int32)
            off_p = self._off.ctypes.data
            nbr_p = self._nbr.ctypes.data if len(self._nbr) else None
            self.n, self.m = len(self._off) - 1, len(self._nbr)
        self.opts = default_opts(**opts)
        h = ctypes.c_void_p()
        _check(L.galp_batch_create(off_p, nbr_p, self.n, self.m, self.graph_v0.ctypes.data, self.count,
                                   ctypes.byref(self.opts), ctypes.byref(h)), "galp_batch_create")
        self._h = h
        self.stats = Stats()

    def run(self, niter: int = 10):
        _check(load_library().galp_run(self._h, niter, ctypes.byref(self.stats)), "galp_run")
        return self.stats.f1, self.stats.f2

    def enqueue(self, niter: int) -> None:
        _check(load_library().galp_enqueue(self._h, niter), "galp_enqueue")

    def sync(self) -> Stats:
        _check(load_library().galp_sync(self._h, ctypes.byref(self.stats)), "galp_sync")
        return self.stats

    def set_stream(self, stream_ptr) -> None:
        _check(load_library().galp_set_stream(self._h, stream_ptr), "galp_set_stream")

    def labels(self, g: int) -> np.ndarray:
        out = np.empty(int(self.graph_v0[g + 1] - self.graph_v0[g]), np.int32)
        _check(load_library().galp_batch_labels(self._h, g, out.ctypes.data if len(out) else None, len(out)),
               "galp_batch_labels")
        return out

    def all_labels(self) -> np.ndarray:
        """Labels of every graph, concatenated in graph order (graph-local values)."""
        out = np.empty(self.n, np.int32)
        _check(load_library().galp_get_labels(self._h, out.ctypes.data if len(out) else None, len(out)),
               "galp_get_labels")
        return out

    def graph_stats(self, g: int):
        """(iterations run, change counts) of graph g in the last run."""
        st = Stats()
        _check(load_library().galp_batch_stats(self._h, g, ctypes.byref(st)), "galp_batch_stats")
        return st.iters_run, [int(x) for x in st.updates[:st.iters_run]]

    def tune(self, niter: int = 3) -> dict:
        from . import tools
        return tools.batch_tune(self, niter)

    def close(self) -> None:
        if getattr(self, "_h", None):
            load_library().galp_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
