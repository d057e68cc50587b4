"""galp_run_noalloc: label propagation without any device allocation.

Callers that cannot call cudaMalloc (an external allocator or host framework owns all
device memory, or an allocation's synchronisation is not acceptable on their path) use
galp_run_noalloc, whose buffers live in a static device array inside the library.  This
test calls it through the C ABI and checks that its labels, iteration count and change
counts equal those of the allocating entry points (galp_create + galp_run +
galp_get_labels) exactly, over consecutive calls that reuse the shared array with
graphs of different sizes.  It lives in its own file so that pytest collects it last.
"""
import ctypes

import numpy as np
import pytest

import galp_gb300

pytestmark = pytest.mark.gpu


def _noalloc():
    L = galp_gb300.load_library()
    L.galp_run_noalloc.argtypes = [ctypes.POINTER(galp_gb300._Csr), ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                   ctypes.POINTER(galp_gb300.Stats), ctypes.c_void_p]
    L.galp_run_noalloc.restype = ctypes.c_int
    return L


def _run_noalloc(g, niter):
    L = _noalloc()
    off = np.ascontiguousarray(g.offsets, dtype=np.int64)
    nbr = np.ascontiguousarray(g.neighbors, dtype=np.int32)
    csr = galp_gb300._Csr(nbr.ctypes.data if len(nbr) else None, off.ctypes.data, len(off) - 1, len(nbr))
    out = np.full(len(off) - 1, -1, np.int32)
    st = galp_gb300.Stats()
    rc = L.galp_run_noalloc(ctypes.byref(csr), niter, 1, out.ctypes.data if len(out) else None, ctypes.byref(st),
                            None)
    assert rc == 0, rc
    return out, st.iters_run, list(st.updates[: st.iters_run])


def _run_allocating(g, niter):
    with galp_gb300.Propagator(g) as p:
        p.run(niter)
        return p.get_labels(), p.iters_run, list(p.updates)


def test_noalloc_matches_allocating_path_on_consecutive_calls():
    big = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=1)        # n = 16,384, m = 295 K
    small = galp_gb300.generate_lfr(3000, seed=7)                        # smaller: stale data must not leak
    hubs = galp_gb300.generate_rmat(13, 8, seed=5)                        # degrees up to a few hundred
    for g in (big, small, big, hubs, small):
        got = _run_noalloc(g, 10)
        want = _run_allocating(g, 10)
        assert got[1] == want[1] and got[2] == want[2]
        assert np.array_equal(got[0], want[0])


def test_noalloc_rejects_graphs_beyond_its_limits():
    L = _noalloc()
    n = (1 << 17) + 1
    off = np.zeros(n + 1, np.int64)
    csr = galp_gb300._Csr(None, off.ctypes.data, n, 0)
    out = np.zeros(n, np.int32)
    assert L.galp_run_noalloc(ctypes.byref(csr), 10, 1, out.ctypes.data, None, None) == -6
