"""CPU oracle for galp's method-0 label-propagation update -- TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py may use this
package, and only as the checker or the timed CPU baseline.  The product path
(galp_gb300) never imports it.

Contents
  lp_oracle.c          literal restatement of DPPBase::perform_lp and the segmented
                       arg-max (reference: src/dpp/dpp.cuh, src/dpp/kernel.cuh,
                       src/common/segmented_reduce.cuh) + the closed form of its tie rule
  lp_oracle_par.cpp    the closed form, multi-threaded, for billion-entry graphs
  cpu_worker_port.cpp  port of the reference's CPU label update CPUWorker::update_label
                       (src/common/hybrid_cpu_worker.cuh:172-195), the timed CPU baseline
  refsim/              the reference's own kernels executed on the CPU (oracle/_ref/)

Parity pinning: the literal restatement is compared bit for bit with the reference's
kernels run through refsim (tests/test_oracle.py) and with the committed golden
vectors in tests/golden/, which refsim generated.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_lib = None
_port = None

REF_HARNESS = os.path.join(HERE, "_ref", "ref_harness")


def _load():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "_build", "liblp_oracle.so")
        if not os.path.exists(path):
            raise RuntimeError(f"oracle not built: {path}")
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.oracle_run.restype = ctypes.c_int64
        L.oracle_run.argtypes = [ctypes.c_int64, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                 ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
        L.oracle_seg_reduce_check.restype = ctypes.c_int
        L.oracle_seg_reduce_check.argtypes = [P, ctypes.c_int64, P, ctypes.c_int64, ctypes.c_int, ctypes.c_int, P, P]
        L.oracle_batch_boundaries.restype = ctypes.c_int64
        L.oracle_batch_boundaries.argtypes = [ctypes.c_int64, P, ctypes.c_int, P, ctypes.c_int64]
        L.oracle_cf_winner.restype = ctypes.c_int64
        L.oracle_cf_winner.argtypes = [P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int]
        L.oracle_step_par.restype = ctypes.c_int64
        L.oracle_step_par.argtypes = [ctypes.c_int64, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                      P, ctypes.c_int]
        L.oracle_run_par.restype = ctypes.c_int64
        L.oracle_run_par.argtypes = [ctypes.c_int64, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                     ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int]
        L.oracle_par_threads.restype = ctypes.c_int
        L.oracle_par_threads.argtypes = []
        _lib = L
    return _lib


def run(offsets, neighbors, niter: int, policy: int = 0, buffer_pow: int = 24, literal: bool = False,
        early_exit: bool = True, TB: int = 256, ET: int = 17):
    """Labels after up to niter iterations.  Returns (iters_run, labels int32[n], counts int64[iters])."""
    L = _load()
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    nbr = np.ascontiguousarray(neighbors, dtype=np.int32)
    n = len(off) - 1
    lab = np.zeros(max(n, 1), np.int32)
    cnt = np.zeros(max(niter, 1), np.int64)
    it = L.oracle_run(n, off.ctypes.data, nbr.ctypes.data, niter, policy, buffer_pow, int(literal), TB, ET,
                      int(bool(early_exit)), lab.ctypes.data, cnt.ctypes.data)
    if it < 0:
        raise RuntimeError(f"oracle_run failed ({it})")
    return int(it), lab[:n].copy(), cnt[:it].copy()


def run_par(offsets, neighbors, niter: int, policy: int = 0, buffer_pow: int = 24, early_exit: bool = True,
            labels=None, threads: int = 0, TB: int = 256, ET: int = 17):
    """Multi-threaded closed form (lp_oracle_par.cpp), same results as run(): labels after
    up to niter iterations starting from vertex IDs, or from `labels` when given.
    Returns (iters_run, labels int32[n], counts int64[iters])."""
    L = _load()
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    nbr = np.ascontiguousarray(neighbors, dtype=np.int32)
    n = len(off) - 1
    lab = np.zeros(max(n, 1), np.int32)
    if labels is not None:
        lab[:n] = np.asarray(labels, np.int32)
    cnt = np.zeros(max(niter, 1), np.int64)
    it = L.oracle_run_par(n, off.ctypes.data, nbr.ctypes.data if len(nbr) else None, niter, policy, buffer_pow, TB,
                          ET, int(bool(early_exit)), int(labels is None), lab.ctypes.data, cnt.ctypes.data, threads)
    if it < 0:
        raise RuntimeError(f"oracle_run_par failed ({it})")
    return int(it), lab[:n].copy(), cnt[:it].copy()


def step_par(offsets, neighbors, labels, policy: int = 0, buffer_pow: int = 24, threads: int = 0,
             TB: int = 256, ET: int = 17):
    """One iteration from the given labels (multi-threaded closed form).
    Returns (new labels int32[n], change count)."""
    L = _load()
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    nbr = np.ascontiguousarray(neighbors, dtype=np.int32)
    n = len(off) - 1
    lab = np.array(labels, dtype=np.int32, copy=True)
    c = L.oracle_step_par(n, off.ctypes.data, nbr.ctypes.data if len(nbr) else None, policy, buffer_pow, TB, ET,
                          lab.ctypes.data if n else None, threads)
    if c < 0:
        raise RuntimeError(f"oracle_step_par failed ({c})")
    return lab, int(c)


def par_threads() -> int:
    return int(_load().oracle_par_threads())


def seg_reduce_check(weights, seg_start, TB: int, ET: int):
    """Literal segmented reduce vs the closed form: (literal_winner[M], closed_form_winner[M])."""
    L = _load()
    w = np.ascontiguousarray(weights, dtype=np.int32)
    s = np.ascontiguousarray(seg_start, dtype=np.int64)
    lit = np.zeros(len(s), np.int64)
    cf = np.zeros(len(s), np.int64)
    rc = L.oracle_seg_reduce_check(w.ctypes.data, len(w), s.ctypes.data, len(s), TB, ET, lit.ctypes.data,
                                   cf.ctypes.data)
    if rc:
        raise RuntimeError("seg_reduce_check failed")
    return lit, cf


def cf_winner(weights, a: int, b: int, N: int, TB: int = 256, ET: int = 17) -> int:
    w = np.ascontiguousarray(weights, dtype=np.int32)
    return int(_load().oracle_cf_winner(w.ctypes.data, a, b, N, TB, ET))


def batch_boundaries(offsets, buffer_pow: int):
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    n = len(off) - 1
    out = np.zeros(n + 2, np.int64)
    nb = _load().oracle_batch_boundaries(n, off.ctypes.data, buffer_pow, out.ctypes.data, n + 2)
    if nb < 0:
        return nb, None
    return nb, out[: nb + 1].copy()


# ---------------------------------------------------------------------------
# the reference's own kernels on the CPU (oracle/_ref/ref_harness)
# ---------------------------------------------------------------------------

def ref_available() -> bool:
    return os.path.exists(REF_HARNESS)


def ref_run(graph_file: str, niter: int, policy: int = 0, buffer_pow: int = 0):
    """Run the reference kernels; returns (per-iteration labels [iters, n], exact counts)."""
    with tempfile.TemporaryDirectory() as td:
        lo, co = os.path.join(td, "l.bin"), os.path.join(td, "c.txt")
        subprocess.run([REF_HARNESS, "lp", graph_file, str(policy), str(buffer_pow), str(niter), lo, co],
                       check=True, stdout=subprocess.DEVNULL)
        counts = np.array([int(x) for x in open(co).read().split()], np.int64)
        lab = np.fromfile(lo, dtype=np.int32)
    iters = len(counts)
    return lab.reshape(iters, -1) if iters else lab.reshape(0, 0), counts


def ref_segreduce(weights, seg_start, TB: int, ET: int) -> np.ndarray:
    w = np.ascontiguousarray(weights, dtype=np.int32)
    s = np.ascontiguousarray(seg_start, dtype=np.int32)
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fi, "wb") as f:
            f.write(np.array([len(w), len(s)], np.int64).tobytes())
            f.write(w.tobytes())
            f.write(s.tobytes())
        subprocess.run([REF_HARNESS, "segreduce", str(TB), str(ET), fi, fo], check=True)
        return np.fromfile(fo, dtype=np.int32)


# ---------------------------------------------------------------------------
# CPU baseline: port of CPUWorker::update_label driven as hybrid_cpu_worker.cuh:123-129
# ---------------------------------------------------------------------------

def _load_port():
    global _port
    if _port is None:
        path = os.path.join(HERE, "_build", "libcpu_worker_port.so")
        if not os.path.exists(path):
            raise RuntimeError(f"CPU worker port not built: {path}")
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        L.cpu_lp_run.restype = ctypes.c_int64
        L.cpu_lp_run.argtypes = [ctypes.c_int64, P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_int,
                                 P, P, ctypes.POINTER(ctypes.c_double)]
        L.cpu_lp_run_strided.restype = ctypes.c_int64
        L.cpu_lp_run_strided.argtypes = [ctypes.c_int64, P, P, ctypes.c_int64, ctypes.c_int64, ctypes.c_int64,
                                         ctypes.c_int, P, P, ctypes.POINTER(ctypes.c_double),
                                         ctypes.POINTER(ctypes.c_int64)]
        L.cpu_lp_threads.restype = ctypes.c_int
        L.cpu_lp_threads.argtypes = []
        _port = L
    return _port


def cpu_baseline(offsets, neighbors, niter: int, v_begin: int = 0, v_end: int | None = None, threads: int = 0):
    """Time niter sweeps of the reference's CPU update over vertices [v_begin, v_end).

    Returns (seconds, threads_used, labels, counts)."""
    L = _load_port()
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    nbr = np.ascontiguousarray(neighbors, dtype=np.int32)
    n = len(off) - 1
    v_end = n if v_end is None else v_end
    lab = np.zeros(max(n, 1), np.int32)
    cnt = np.zeros(max(niter, 1), np.int64)
    secs = ctypes.c_double()
    used = L.cpu_lp_run(n, off.ctypes.data, nbr.ctypes.data, v_begin, v_end, niter, threads, lab.ctypes.data,
                        cnt.ctypes.data, ctypes.byref(secs))
    return secs.value, int(used), lab[:n], cnt[:niter]


def cpu_baseline_strided(offsets, neighbors, niter: int, stride: int, phase: int = 0, threads: int = 0):
    """Time niter in-place sweeps of the reference's CPU update over the strided vertex
    sample phase, phase + stride, ...  Returns (seconds, threads_used, sample CSR entries,
    counts)."""
    L = _load_port()
    off = np.ascontiguousarray(offsets, dtype=np.int64)
    nbr = np.ascontiguousarray(neighbors, dtype=np.int32)
    n = len(off) - 1
    lab = np.zeros(max(n, 1), np.int32)
    cnt = np.zeros(max(niter, 1), np.int64)
    secs = ctypes.c_double()
    edges = ctypes.c_int64()
    used = L.cpu_lp_run_strided(n, off.ctypes.data, nbr.ctypes.data, stride, phase, niter, threads, lab.ctypes.data,
                                cnt.ctypes.data, ctypes.byref(secs), ctypes.byref(edges))
    return secs.value, int(used), int(edges.value), cnt[:niter]
