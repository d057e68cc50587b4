"""Hubs (vertices above 12288 neighbours, counted in global tables by chunks of 1024 edges):
labels, change counts and iteration counts equal the oracle after every iteration for hubs of
25,000-80,000 neighbours joined to whole planted communities, from the first iterations, where
a hub's labels are nearly all distinct and repeat across its chunks, to the last, where its
neighbours share one or two labels (aggregated inserts, heavily repeated merges), under every
insert-aggregation mode and with the frontier."""
import numpy as np
import pytest

import galp_gb300
import oracle
from galp_gb300 import tools

pytestmark = pytest.mark.gpu

SIZES = [20000, 20000, 10000, 15000, 15000]   # planted communities
HUBS = [[0, 1, 2], [3, 4, 2], [0, 1, 2, 3, 4], [2, 3], [0, 3]]  # communities each hub joins


def _graph(seed):
    """Hubs take the smallest IDs; the communities follow, each vertex with about 8 random
    neighbours inside its community and one edge to every hub that joins its community."""
    rng = np.random.default_rng(seed)
    nh = len(HUBS)
    starts = nh + np.concatenate([[0], np.cumsum(SIZES)])
    src, dst = [], []
    for c, size in enumerate(SIZES):
        src.append(rng.integers(0, size, 4 * size) + starts[c])
        dst.append(rng.integers(0, size, 4 * size) + starts[c])
    n = int(starts[-1])
    for h, cs in enumerate(HUBS):
        members = np.concatenate([np.arange(starts[c], starts[c + 1]) for c in cs])
        src.append(np.full(len(members), h))
        dst.append(members)
    s = np.concatenate(src)
    d = np.concatenate(dst)
    keep = s != d
    s, d = s[keep], d[keep]
    pairs = np.unique(np.stack([np.concatenate([s, d]), np.concatenate([d, s])], 1), axis=0)
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, pairs[:, 0] + 1, 1)
    return galp_gb300.Graph(np.cumsum(off), pairs[:, 1].astype(np.int32))


@pytest.fixture(scope="module")
def hub_graph():
    g = _graph(seed=17)
    deg = g.degrees()
    assert (deg[:len(HUBS)] > 12288).all()  # the hub path, several chunks each
    return g


def _check_every_iteration(g, niter, agg=None, **opts):
    """Labels, change counts and iteration counts after each of the first niter iterations
    equal the oracle's (both stop early under the same rule)."""
    with galp_gb300.Propagator(g, **opts) as p:
        if agg is not None:
            tools.set_variant(p, agg_mode=agg)
        for k in range(1, niter + 1):
            p.run(k)
            got = p.get_labels()
            it, want, counts = oracle.run(g.offsets, g.neighbors, k)
            assert p.iters_run == it, f"run({k}): {p.iters_run} iterations vs oracle {it}"
            assert np.array_equal(got, want), f"run({k}): {np.count_nonzero(got != want)} labels differ"
            assert list(p.updates) == list(counts), f"run({k}): change counts differ"
            if it < k:
                break


@pytest.mark.parametrize("agg", [None, 1, 2])
def test_hubs_every_iteration(hub_graph, agg):
    _check_every_iteration(hub_graph, 10, agg=agg)


def test_hubs_with_frontier(hub_graph):
    _check_every_iteration(hub_graph, 10, frontier=1)


def _spread_hubs(g, nh):
    """The same graph with the hubs (IDs 0..nh-1) moved to evenly spaced IDs, so that under
    out-of-core batching they sit inside later batches, at nonzero batch-local run positions."""
    n = g.n
    pos = np.array([(h + 1) * n // (nh + 1) for h in range(nh)])
    rest = np.setdiff1d(np.arange(n), pos)
    perm = np.empty(n, np.int64)  # old ID -> new ID
    perm[:nh] = pos
    perm[nh:] = rest
    src = np.repeat(perm, g.degrees())
    dst = perm[g.neighbors]
    order = np.lexsort((dst, src))
    off = np.zeros(n + 1, np.int64)
    np.add.at(off, src + 1, 1)
    return galp_gb300.Graph(np.cumsum(off), dst[order].astype(np.int32)), pos


@pytest.mark.parametrize("policy", [1, 2])
@pytest.mark.parametrize("bpow", [17, 18])
def test_hubs_inside_out_of_core_batches(hub_graph, policy, bpow):
    g, pos = _spread_hubs(hub_graph, len(HUBS))
    deg = g.degrees()
    assert (deg[pos] > 12288).all()
    nb, bbs = oracle.batch_boundaries(g.offsets, bpow)
    assert nb > 1
    hub_batches = set(np.searchsorted(bbs, pos, side="right") - 1)
    assert len(hub_batches - {0}) >= 1  # at least one hub in a batch after the first
    with galp_gb300.Propagator(g, policy=policy, buffer_pow=bpow) as p:
        for k in range(1, 11):
            p.run(k)
            it, want, counts = oracle.run(g.offsets, g.neighbors, k, policy=policy, buffer_pow=bpow)
            assert p.iters_run == it
            got = p.get_labels()
            assert np.array_equal(got, want), f"run({k}): {np.count_nonzero(got != want)} labels differ"
            assert list(p.updates) == list(counts)
            if it < k:
                break


@pytest.mark.parametrize("shift", [-6, 0, 2])
def test_hub_partition_count_does_not_change_labels(hub_graph, shift):
    """Hubs count their labels in degree * 2^shift / 8192 hash partitions.
    With far too few partitions (shift -6: one per hub, whose table holds fewer distinct
    labels than the hub's neighbours carry) the first iterations overflow them; the run is
    redone with twice the partitions until none overflows, and its labels are exact.  The
    other partition sizes, each counted by its own CTA shape (shift 0: 1024 threads, the
    default 1: 512, 2: 256), are exact too."""
    with galp_gb300.Propagator(hub_graph) as p:
        tools.set_variant(p, hub_part_shift=shift)
        for k in (1, 2, 3, 10):
            p.run(k)
            it, want, counts = oracle.run(hub_graph.offsets, hub_graph.neighbors, k)
            assert p.iters_run == it and list(p.updates) == list(counts)
            assert np.array_equal(p.get_labels(), want)
            if it < k:
                break
        v = tools.set_variant(p)
        if shift < 0:
            assert v.hub_part_shift > shift  # overflowed at least once and was redone
        else:
            assert v.hub_part_shift == shift
