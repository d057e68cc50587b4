"""Frontier mode (opts.frontier = 1): vertices whose neighbour labels did not change carry
their counts and summaries over; labels and change counts must still equal the oracle's
after every iteration, and asymmetric graphs must fall back to the dense update."""
import numpy as np
import pytest

import galp_gb300
import oracle
from galp_gb300 import tools

pytestmark = pytest.mark.gpu


def _check_every_iteration(g, niter, expect_frontier=True, **opts):
    with galp_gb300.Propagator(g, frontier=1, **opts) as p:
        info = tools.schedule_info(p)
        assert bool(info.flags & tools.SchedInfo.FRONTIER) == expect_frontier
        for k in range(1, niter + 1):
            p.run(k)
            got = p.get_labels()
            it, want, counts = oracle.run(g.offsets, g.neighbors, k, policy=opts.get("policy", 0),
                                          buffer_pow=opts.get("buffer_pow", 24))
            assert p.iters_run == it, f"run({k}): {p.iters_run} iterations vs oracle {it}"
            assert np.array_equal(got, want), f"run({k}): {np.count_nonzero(got != want)} labels differ"
            assert list(p.updates) == list(counts), f"run({k}): change counts differ"
            if it < k:
                break


def _csr(n, src, dst):
    order = np.lexsort((dst, src))
    src, dst = src[order], dst[order]
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, src + 1, 1)
    return galp_gb300.Graph(np.cumsum(off), dst.astype(np.int32))


def _bipartite(sizes):
    src, dst, base = [], [], 0
    for a, b in sizes:
        s = np.repeat(np.arange(base, base + a), b)
        d = np.tile(np.arange(base + a, base + a + b), a)
        src += [s, d]
        dst += [d, s]
        base += a + b
    return _csr(base, np.concatenate(src), np.concatenate(dst))


def test_sbm_ten_iterations_no_early_exit():
    g = galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=1)
    with galp_gb300.Propagator(g, frontier=1, early_exit=0) as p:
        p.run(10)
        got, upd = p.get_labels(), list(p.updates)
    with galp_gb300.Propagator(g, early_exit=0) as p:
        p.run(10)
        assert np.array_equal(got, p.get_labels()) and upd == list(p.updates)
    it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
    assert np.array_equal(got, want)


def test_sbm_every_iteration():
    _check_every_iteration(galp_gb300.generate_sbm([256] * 64, 16.0, 2.0, seed=3), 8)


def test_lfr_every_iteration():
    _check_every_iteration(galp_gb300.generate_lfr(20000, seed=5), 8)


def test_rmat_with_hubs():
    _check_every_iteration(galp_gb300.generate_rmat(15, 16, seed=11), 6)
    _check_every_iteration(galp_gb300.generate_rmat(17, 16, seed=11), 4)


def test_ties_in_every_bucket():
    # exact ties at degrees 3..13000: clean tied vertices are re-resolved with moved run bases
    _check_every_iteration(_bipartite([(3, 2), (40, 7), (300, 9), (2500, 40), (13000, 3), (700, 33)]), 5)


def test_unsorted_adjacency():
    g = galp_gb300.generate_lfr(20000, seed=12)
    rng = np.random.default_rng(3)
    nbr = g.neighbors.copy()
    for v in range(g.n):
        lo, hi = g.offsets[v], g.offsets[v + 1]
        nbr[lo:hi] = rng.permutation(nbr[lo:hi])
    g2 = galp_gb300.Graph(g.offsets, nbr)
    with galp_gb300.Propagator(g2, frontier=1) as p:
        f = tools.schedule_info(p).flags
    assert not (f & tools.SchedInfo.SORTED) and (f & tools.SchedInfo.SYMMETRIC)
    _check_every_iteration(g2, 5)


def test_asymmetric_graph_runs_dense():
    # a directed graph: marking along out-edges would miss in-neighbours, so the frontier
    # must switch itself off (and the labels still follow the oracle)
    rng = np.random.default_rng(7)
    n = 5000
    src = rng.integers(0, n, 60000)
    dst = rng.integers(0, n, 60000)
    keep = src != dst
    pairs = np.unique(np.stack([src[keep], dst[keep]], 1), axis=0)
    g = _csr(n, pairs[:, 0], pairs[:, 1])
    with galp_gb300.Propagator(g, frontier=1) as p:
        f = tools.schedule_info(p).flags
    assert f & tools.SchedInfo.SORTED and not (f & tools.SchedInfo.SYMMETRIC)
    _check_every_iteration(g, 5, expect_frontier=False)


def test_single_missing_reverse_edge_detected():
    g = galp_gb300.generate_sbm([64] * 16, 8.0, 1.0, seed=9)
    # drop one direction of one edge
    v = int(np.argmax(g.degrees()))
    lo = g.offsets[v]
    nbr = np.delete(g.neighbors, lo)
    off = g.offsets.copy()
    off[v + 1:] -= 1
    g2 = galp_gb300.Graph(off, nbr)
    with galp_gb300.Propagator(g2, frontier=1) as p:
        assert not (tools.schedule_info(p).flags & tools.SchedInfo.SYMMETRIC)
    with galp_gb300.Propagator(g, frontier=1) as p:
        assert tools.schedule_info(p).flags & tools.SchedInfo.FRONTIER


def test_out_of_core_policies_ignore_the_frontier():
    g = galp_gb300.generate_sbm([128] * 32, 10.0, 2.0, seed=4)
    _check_every_iteration(g, 4, expect_frontier=False, policy=2, buffer_pow=12)


def test_launch_count_reported():
    g = galp_gb300.generate_rmat(14, 16, seed=4)
    with galp_gb300.Propagator(g, frontier=1, early_exit=0) as p:
        before = tools.schedule_info(p).launches
        p.run(5)
        info = tools.schedule_info(p)
        assert 0 < info.launches - before <= 4 + 5 * info.launches_per_iter


@pytest.mark.parametrize("frac", [0.0, 0.05, 1.0])
def test_frontier_switch_threshold(frac):
    # 0: every iteration recounts all vertices (the device switches the frontier off);
    # 1: the frontier is used whenever it is available
    g = galp_gb300.generate_rmat(15, 16, seed=2)
    with galp_gb300.Propagator(g, frontier=1) as p:
        tools.set_variant(p, frontier_frac=frac)
        p.run(8)
        got, upd, its = p.get_labels(), list(p.updates), p.iters_run
    it, want, counts = oracle.run(g.offsets, g.neighbors, 8)
    assert its == it and np.array_equal(got, want) and upd == list(counts)


@pytest.mark.parametrize("agg", [0, 1, 2])
def test_insert_aggregation_variants(agg):
    g = galp_gb300.generate_rmat(16, 16, seed=5)
    with galp_gb300.Propagator(g) as p:
        tools.set_variant(p, agg_mode=agg)
        p.run(6)
        got, its = p.get_labels(), p.iters_run
    it, want, counts = oracle.run(g.offsets, g.neighbors, 6)
    assert its == it and np.array_equal(got, want)


@pytest.mark.parametrize("small_sort", [0, 1, 2])
def test_small_pack_counting_variants(small_sort):
    # sort-based and match-based counting of small-vertex packs, and one thread per small
    # vertex, give the same labels, with the frontier too
    for g in (galp_gb300.generate_rmat(16, 8, seed=6), galp_gb300.generate_lfr(20000, seed=8),
              galp_gb300.generate_sbm([128] * 32, 10.0, 3.0, seed=2)):
        it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
        for fr in (0, 1):
            with galp_gb300.Propagator(g, frontier=fr) as p:
                tools.set_variant(p, small_sort=small_sort)
                p.run(10)
                got, its, upd = p.get_labels(), p.iters_run, list(p.updates)
            assert its == it and upd == list(counts) and np.array_equal(got, want)


@pytest.mark.parametrize("small_sort", [0, 2])
def test_small_counting_variants_out_of_core_and_isolated(small_sort):
    # isolated vertices among the small ones, and out-of-core batches (small-vertex lists
    # per batch)
    g = galp_gb300.generate_sbm([64] * 16, 8.0, 2.0, seed=9)
    new_n = g.n + 4
    iso = np.array([0, 3, 500, new_n - 1])
    keep = np.setdiff1d(np.arange(new_n), iso)
    deg = np.zeros(new_n, np.int64)
    deg[keep] = g.degrees()
    off = np.zeros(new_n + 1, np.int64)
    off[1:] = np.cumsum(deg)
    g2 = galp_gb300.Graph(off, keep[g.neighbors].astype(np.int32))
    for opts in ({}, {"policy": 2, "buffer_pow": 11}):
        it, want, counts = oracle.run(g2.offsets, g2.neighbors, 10, policy=opts.get("policy", 0),
                                      buffer_pow=opts.get("buffer_pow", 24))
        with galp_gb300.Propagator(g2, **opts) as p:
            tools.set_variant(p, small_sort=small_sort)
            p.run(10)
            assert p.iters_run == it and list(p.updates) == list(counts)
            assert np.array_equal(p.get_labels(), want)


@pytest.mark.parametrize("mid_sort", [0, 1])
def test_sort_reduce_mid_counting_variant(mid_sort):
    # vertices of 33..256 neighbours counted by hash tables or by a warp bitonic sort and
    # run detection (the method-0 way): the same labels and change counts, dense and with
    # the frontier, in-core and out of core, with every warp/CTA split of the variant rows
    for g in (galp_gb300.generate_rmat(16, 16, seed=6), galp_gb300.generate_lfr(20000, seed=8),
              galp_gb300.generate_sbm([128] * 32, 40.0, 8.0, seed=2)):
        assert ((g.degrees() > 32) & (g.degrees() <= 256)).sum() > 500
        it, want, counts = oracle.run(g.offsets, g.neighbors, 10)
        for fr in (0, 1):
            with galp_gb300.Propagator(g, frontier=fr) as p:
                tools.set_variant(p, mid_sort=mid_sort)
                p.run(10)
                assert p.iters_run == it and list(p.updates) == list(counts)
                assert np.array_equal(p.get_labels(), want)
    g = galp_gb300.generate_rmat(15, 16, seed=11)
    for row in (0, 2, 4, 6):
        with galp_gb300.Propagator(g, frontier=1) as p:
            tools.dispatch_set(p, 2, row)
            tools.set_variant(p, mid_sort=mid_sort)
            p.run(8)
            it, want, counts = oracle.run(g.offsets, g.neighbors, 8)
            assert p.iters_run == it and np.array_equal(p.get_labels(), want)
    it, want, counts = oracle.run(g.offsets, g.neighbors, 5, policy=2, buffer_pow=14)
    with galp_gb300.Propagator(g, policy=2, buffer_pow=14) as p:
        tools.set_variant(p, mid_sort=mid_sort)
        p.run(5)
        assert p.iters_run == it and list(p.updates) == list(counts)
        assert np.array_equal(p.get_labels(), want)
