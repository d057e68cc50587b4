"""GPU parity: the sm_103a update through the C ABI vs the CPU oracle, bit for bit."""
import numpy as np
import pytest

import galp_gb300
import oracle

pytestmark = pytest.mark.gpu


def _gpu_run(g, niter, **opts):
    with galp_gb300.Propagator(g, **opts) as p:
        p.run(niter)
        return p.iters_run, p.get_labels(), np.array(p.updates, np.int64)


def _check_every_iteration(g, niter, **opts):
    """Labels and change counts after each of the first niter iterations equal the oracle's
    (both stop early under the same rule, so their iteration counts must agree too)."""
    with galp_gb300.Propagator(g, **opts) as p:
        for k in range(1, niter + 1):
            p.run(k)
            got = p.get_labels()
            it, want, counts = oracle.run(g.offsets, g.neighbors, k)
            assert p.iters_run == it, f"run({k}): {p.iters_run} iterations vs oracle {it}"
            assert np.array_equal(got, want), f"run({k}): {np.count_nonzero(got != want)} labels differ"
            assert list(p.updates) == list(counts), f"run({k}): change counts differ"
            if it < k:
                break


def test_sample_graph():
    # datasets/sample.txt of the reference: 7 vertices, 9 undirected edges
    edges = [(0, 1), (0, 2), (1, 2), (2, 3), (3, 4), (3, 5), (4, 5), (4, 6), (5, 6)]
    adj = [[] for _ in range(7)]
    for u, v in edges:
        adj[u].append(v)
        adj[v].append(u)
    off = np.zeros(8, np.int64)
    off[1:] = np.cumsum([len(a) for a in adj])
    nbr = np.array([x for a in adj for x in a], np.int32)
    g = galp_gb300.Graph(off, nbr)
    _check_every_iteration(g, 6)


def test_sbm_config_10_iterations():
    # planted partition: n = 16,384, 64 blocks of 256, expected degrees 16 / 2
    g = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=1)
    it, got, upd = _gpu_run(g, 10)
    want_it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
    assert it == want_it
    assert np.array_equal(upd, counts)
    assert np.array_equal(got, want)


def test_sbm_every_iteration():
    g = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=3)
    _check_every_iteration(g, 5)


@pytest.mark.parametrize("method", [0, 1])
def test_lfr_small(method):
    g = galp_gb300.generate_lfr(20000, seed=5)
    it, got, upd = _gpu_run(g, 10, method=method)
    want_it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
    assert it == want_it and np.array_equal(upd, counts)
    assert np.array_equal(got, want)


def test_rmat_with_hubs():
    # scale 15: degree-1 vertices up to hubs of a few thousand (every counting bucket
    # below the global tables); scale 17: one hub above 12288 (global-table path)
    g = galp_gb300.generate_rmat(15, 16, seed=11)
    assert g.degrees().max() > 2048
    _check_every_iteration(g, 4)
    g = galp_gb300.generate_rmat(17, 16, seed=11)
    assert g.degrees().max() > 12288
    _check_every_iteration(g, 3)


def _bipartite(sizes):
    """Disjoint complete bipartite blocks K(a, b): many exact ties at every degree."""
    src, dst, base = [], [], 0
    for a, b in sizes:
        left = np.arange(base, base + a)
        right = np.arange(base + a, base + a + b)
        s = np.repeat(left, b)
        d = np.tile(right, a)
        src += [s, d]
        dst += [d, s]
        base += a + b
    src, dst = np.concatenate(src), np.concatenate(dst)
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(base + 1, np.int64)
    np.add.at(off, src + 1, 1)
    return galp_gb300.Graph(np.cumsum(off), dst.astype(np.int32))


def test_xl_and_global_table_ties():
    # right sides of degree 2500 (one CTA, 192 KB table) and 13000 (global table)
    g = _bipartite([(2500, 40), (13000, 3), (5000, 5)])
    _check_every_iteration(g, 3)


def test_unsorted_adjacency():
    # adjacency lists in arbitrary order: the first iteration takes the general path
    g = galp_gb300.generate_lfr(20000, seed=12)
    rng = np.random.default_rng(3)
    nbr = g.neighbors.copy()
    for v in range(g.n):
        lo, hi = g.offsets[v], g.offsets[v + 1]
        nbr[lo:hi] = rng.permutation(nbr[lo:hi])
    _check_every_iteration(galp_gb300.Graph(g.offsets, nbr), 3)


def test_mid_degree_ties():
    # vertices of degree 40..1500 whose neighbours carry few distinct labels, with
    # many exact ties: complete bipartite blocks force equal counts
    rng = np.random.default_rng(0)
    blocks = []
    base = 0
    for size in [40, 90, 300, 700, 1500, 33, 64, 2000]:
        left = np.arange(base, base + size)
        right = np.arange(base + size, base + 2 * size)
        blocks.append((left, right))
        base += 2 * size
    n = base
    src, dst = [], []
    for left, right in blocks:
        s = np.repeat(left, len(right))
        d = np.tile(right, len(left))
        src += [s, d]
        dst += [d, s]
    src = np.concatenate(src)
    dst = np.concatenate(dst)
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, src + 1, 1)
    off = np.cumsum(off)
    g = galp_gb300.Graph(off, dst.astype(np.int32))
    _check_every_iteration(g, 3)
    del rng


def test_isolated_vertices_keep_their_label():
    g = galp_gb300.generate_sbm([64] * 8, 6.0, 1.0, seed=2)
    # insert isolated vertices at the front, the middle and the end
    n = g.n
    deg = g.degrees()
    iso = [0, n // 2, n + 2]
    new_n = n + len(iso)
    keep = np.setdiff1d(np.arange(new_n), iso)
    remap = np.full(n, -1, np.int64)
    remap[:] = keep
    new_deg = np.zeros(new_n, np.int64)
    new_deg[keep] = deg
    off = np.zeros(new_n + 1, np.int64)
    off[1:] = np.cumsum(new_deg)
    nbr = remap[g.neighbors].astype(np.int32)
    g2 = galp_gb300.Graph(off, nbr)
    it, got, upd = _gpu_run(g2, 10)
    want_it, want, counts = oracle.run(g2.offsets, g2.neighbors, 10)  # closed form defines degree 0
    assert it == want_it and np.array_equal(got, want)
    for v in iso:
        assert got[v] == v


def test_empty_and_tiny_graphs():
    g = galp_gb300.Graph(np.zeros(1, np.int64), np.zeros(0, np.int32))
    it, got, upd = _gpu_run(g, 10)
    assert len(got) == 0
    g = galp_gb300.Graph(np.array([0, 1, 2], np.int64), np.array([1, 0], np.int32))
    it, got, upd = _gpu_run(g, 10)
    want_it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
    assert np.array_equal(got, want) and it == want_it


def test_malformed_graph_rejected():
    off = np.array([0, 1, 2], np.int64)
    nbr = np.array([1, 5], np.int32)  # 5 is out of range
    with pytest.raises(galp_gb300.GalpError) as e:
        galp_gb300.Propagator(galp_gb300.Graph(off, nbr))
    assert e.value.code == -5


def test_deterministic_repeat():
    g = galp_gb300.generate_rmat(14, 16, seed=4)
    a = _gpu_run(g, 10)[1]
    b = _gpu_run(g, 10)[1]
    assert np.array_equal(a, b)
