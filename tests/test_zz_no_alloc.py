"""galp_run_noalloc: label propagation without any device allocation.

Callers that cannot call cudaMalloc (an external allocator or host framework owns all
device memory, or an allocation's synchronisation is not acceptable on their path) use
galp_run_noalloc, whose buffers live in a static device array inside the library.  These
tests call it through the C ABI and check that its labels, iteration count and change
counts equal those of the allocating entry points (galp_create + galp_run +
galp_get_labels) exactly, over consecutive calls that reuse the shared array with
graphs of different sizes; that they equal the oracle directly (it runs a different
kernel from galp_run), at its documented limits and with fixed iteration counts; that
graphs beyond the limits are rejected; and that a look-back wait that runs out ends
the call with GALP_ETIMEOUT instead of a hang, after which the next call is exact
again.  They live in their own file so that pytest collects them last.
"""
import ctypes

import numpy as np
import pytest

import galp_gb300
import oracle

pytestmark = pytest.mark.gpu


def _noalloc():
    L = galp_gb300.load_library()
    L.galp_run_noalloc.argtypes = [ctypes.POINTER(galp_gb300._Csr), ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p,
                                   ctypes.POINTER(galp_gb300.Stats), ctypes.c_void_p]
    L.galp_run_noalloc.restype = ctypes.c_int
    return L


def _call(g, niter, early_exit=1):
    L = _noalloc()
    off = np.ascontiguousarray(g.offsets, dtype=np.int64)
    nbr = np.ascontiguousarray(g.neighbors, dtype=np.int32)
    csr = galp_gb300._Csr(nbr.ctypes.data if len(nbr) else None, off.ctypes.data, len(off) - 1, len(nbr))
    out = np.full(len(off) - 1, -1, np.int32)
    st = galp_gb300.Stats()
    rc = L.galp_run_noalloc(ctypes.byref(csr), niter, early_exit, out.ctypes.data if len(out) else None,
                            ctypes.byref(st), None)
    return rc, out, st


def _run_noalloc(g, niter, early_exit=1):
    rc, out, st = _call(g, niter, early_exit)
    assert rc == 0, rc
    return out, st.iters_run, list(st.updates[: st.iters_run])


def _sym_graph(n, src, dst):
    """Symmetric CSR without self-loops or duplicate edges from undirected pairs."""
    src, dst = np.asarray(src, np.int64), np.asarray(dst, np.int64)
    keep = src != dst
    key = np.unique(np.concatenate([src[keep] * n + dst[keep], dst[keep] * n + src[keep]]))
    u, v = key // n, key % n
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, u + 1, 1)
    return galp_gb300.Graph(np.cumsum(off), v.astype(np.int32))


def _check_oracle(g, niter, early_exit=1):
    got, its, upd = _run_noalloc(g, niter, early_exit)
    it, want, counts = oracle.run(g.offsets, g.neighbors, niter, early_exit=bool(early_exit))
    assert its == it and upd == list(counts)
    assert np.array_equal(got, want), f"{np.count_nonzero(got != want)} labels differ"


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


def test_noalloc_equals_the_oracle():
    for g in (galp_gb300.generate_sbm([128] * 32, 12.0, 2.0, seed=3), galp_gb300.generate_lfr(20000, seed=4),
              galp_gb300.generate_rmat(13, 8, seed=9)):
        assert g.degrees().max() <= 2048  # within the entry point's limit
        _check_oracle(g, 10)


def test_noalloc_at_its_limits():
    rng = np.random.default_rng(21)
    # a vertex of exactly 2048 neighbours after a partly filled tile, one of 2047 and one
    # of 2046 at the start of the ID range, over a sparse random graph among the others
    n = 6000
    hubs = {3001: 2048, 100: 2047, 0: 2046}
    rest = np.setdiff1d(np.arange(n), list(hubs))
    src = [rng.choice(rest, 5 * n)]
    dst = [rng.choice(rest, 5 * n)]
    for hub, deg in hubs.items():
        src.append(np.full(deg, hub))
        dst.append(rng.choice(rest, deg, replace=False))
    g = _sym_graph(n, np.concatenate(src), np.concatenate(dst))
    assert all(g.degrees()[h] == d for h, d in hubs.items())
    _check_oracle(g, 10)
    # the largest graph it accepts: n = 2^17 vertices, m just below 2^21 entries
    n = 1 << 17
    a = rng.integers(0, n, 1 << 21)
    b = rng.integers(0, n, 1 << 21)
    key = np.unique(np.minimum(a, b)[a != b] * n + np.maximum(a, b)[a != b])
    key = rng.permutation(key)[:(1 << 20) - 64]
    g = _sym_graph(n, key // n, key % n)
    assert g.n == n and g.m == (1 << 21) - 128
    _check_oracle(g, 10)


def test_noalloc_fixed_iteration_counts():
    g = galp_gb300.generate_sbm([64] * 8, 10.0, 0.5, seed=4)
    out, its, upd = _run_noalloc(g, 0, early_exit=0)
    assert its == 0 and upd == [] and np.array_equal(out, np.arange(g.n, dtype=np.int32))
    _check_oracle(g, 30, early_exit=0)  # runs past convergence: zero changes, same labels
    _check_oracle(g, 30, early_exit=1)


def test_noalloc_rejects_m_and_degree_beyond_the_limits():
    L = _noalloc()
    m = (1 << 21) + 1
    off = np.array([0, m], np.int64)
    nbr = np.zeros(m, np.int32)
    csr = galp_gb300._Csr(nbr.ctypes.data, off.ctypes.data, 1, m)
    out = np.zeros(1, np.int32)
    assert L.galp_run_noalloc(ctypes.byref(csr), 10, 1, out.ctypes.data, None, None) == -6
    star = _sym_graph(2050, np.zeros(2049, np.int64), np.arange(1, 2050))
    assert star.degrees()[0] == 2049
    rc, _, _ = _call(star, 10)
    assert rc == -6


def test_noalloc_lookback_timeout_is_reported_and_recovers():
    """Failure detection without a GPU fault: the test hook makes every look-back wait
    expect a status no tile publishes, with a short poll limit; the kernel gives up,
    returns, and the call reports GALP_ETIMEOUT (-4).  With the hook cleared, the next
    calls are exact again."""
    L = _noalloc()
    L.galp_debug_noalloc_lookback.argtypes = [ctypes.c_int64, ctypes.c_int32]
    L.galp_debug_noalloc_lookback.restype = ctypes.c_int
    g = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=1)  # many tiles: every tile after the first waits
    assert L.galp_debug_noalloc_lookback(2000, 1) == 0
    try:
        rc, _, st = _call(g, 3)
    finally:
        assert L.galp_debug_noalloc_lookback(0, 0) == 0
    assert rc == -4 and st.err & 1
    _check_oracle(g, 10)
    _check_oracle(galp_gb300.generate_lfr(3000, seed=7), 10)
